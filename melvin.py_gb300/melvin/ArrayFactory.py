"""Array creation with the reference's shapes (melvin/ArrayFactory.py)."""

import torch


class ArrayFactory:
    def __init__(self, params, xp=None):
        self._p = params
        self._xp = xp
        self._device = torch.device(getattr(params, "device", "cuda"))

    def make_mode_number_matrices(self):
        """Integer (n, m) meshgrids (melvin/ArrayFactory.py:8-26)."""
        p = self._p
        kw = dict(device=self._device, dtype=torch.int64)
        if p.is_fully_spectral():
            n = torch.cat((torch.arange(0, p.nn + 1, **kw), torch.arange(-p.nn, 0, **kw)))
            m = torch.arange(0, p.nm, **kw)
        elif p.discretisation[0] == "fdm":
            n = torch.arange(0, p.nx, **kw)
            m = torch.arange(0, p.nm, **kw)
        else:
            n = torch.arange(0, p.nn, **kw)
            m = torch.arange(0, p.nz, **kw)
        return torch.meshgrid(n, m, indexing="ij")

    def make_spectral(self, ni=None, nj=None):
        ni = self._p.spectral_shape[0] if ni is None else ni
        nj = self._p.spectral_shape[1] if nj is None else nj
        return torch.zeros((ni, nj), dtype=torch.complex128, device=self._device)

    def make_physical(self, nx=None, nz=None):
        nx = self._p.nx if nx is None else nx
        nz = self._p.nz if nz is None else nz
        return torch.zeros((nx, nz), dtype=torch.float64, device=self._device)
