"""Conversions between user arrays (numpy, tensors, scalars) and the
contiguous device tensors the native calls take."""

import numpy as np
import torch

from . import _native as N


def as_device(x, dtype, device, shape=None):
    """Contiguous tensor of `dtype` on `device`; no copy when `x` already is one."""
    if isinstance(x, torch.Tensor):
        t = x
        if t.device != device:
            t = t.to(device)
        if t.dtype != dtype:
            if dtype.is_complex or not t.dtype.is_complex:
                t = t.to(dtype)
            else:
                raise TypeError(f"expected a real array, got {t.dtype}")
    else:
        a = np.asarray(x)
        if np.iscomplexobj(a) and not dtype.is_complex:
            raise TypeError(f"expected a real array, got {a.dtype}")
        t = torch.as_tensor(a, device=device).to(dtype)
    if shape is not None and tuple(t.shape) != tuple(shape):
        t = t.expand(shape) if t.dim() == 0 else t
        if tuple(t.shape) != tuple(shape):
            raise ValueError(f"expected shape {tuple(shape)}, got {tuple(t.shape)}")
    return t.contiguous()


def native_target(out, dtype, shape, device):
    """(tensor the native call writes into, out) -- a fresh tensor when `out`
    is None, `out` itself when it is a suitable device tensor, else a scratch
    tensor whose value `finish` copies back into `out`."""
    if out is None:
        t = torch.empty(shape, dtype=dtype, device=device)
        return t, t
    if (
        isinstance(out, torch.Tensor)
        and out.device == device
        and out.dtype == dtype
        and out.is_contiguous()
        and tuple(out.shape) == tuple(shape)
    ):
        return out, out
    return torch.empty(shape, dtype=dtype, device=device), out


def finish(tmp, out):
    if out is tmp:
        return out
    if isinstance(out, torch.Tensor):
        out.copy_(tmp)
        return out
    out[...] = tmp.cpu().numpy()
    return out


def cplx(t):
    return N.ptr(t)
