"""A field with spectral and physical storage (melvin/Variable.py).

``_sdata`` (complex128, spectral shape) and ``_pdata`` (float64, physical
shape) are device tensors.  Indexing reads and writes the spectral data, as
in the reference, so boundary-condition slicing such as ``w[1:, :2] = 0.0``
works unchanged.
"""

import numpy as np
import torch

from . import _native as N
from ._arrays import as_device
from .BasisFunctions import BasisFunctions


class Variable:
    def __init__(self, params, xp=None, sd=None, st=None, dt=None, array_factory=None, dump_name=None,
                 basis_functions=None):
        self._params = params
        self._xp = xp
        self._st = st
        self._sd = sd
        self._dt = dt
        self._array_factory = array_factory
        self._dump_name = dump_name
        if basis_functions is None:
            raise Exception("Basis functions must be specified.")
        self._basis_functions = basis_functions
        self._sdata = array_factory.make_spectral()
        self._pdata = array_factory.make_physical()
        self._device = self._sdata.device

    def __setitem__(self, index, value):
        if isinstance(value, np.ndarray):
            value = torch.as_tensor(value, device=self._device)
        self._sdata[index] = value

    def __getitem__(self, index):
        return self._sdata[index]

    def sets(self, data):
        self._sdata[:, :] = as_device(data, torch.complex128, self._device)

    def setp(self, data):
        self._pdata[:, :] = as_device(data, torch.float64, self._device)

    def getp(self):
        return self._pdata

    def gets(self):
        return self._sdata

    def to_physical(self):
        self._st.to_physical(self._sdata, self._pdata, self._basis_functions)

    def to_spectral(self):
        self._st.to_spectral(self._pdata, self._sdata, self._basis_functions)

    def load(self, data, is_physical=False):
        if isinstance(data, str):
            raise NotImplementedError
        if self._dt is not None:
            data = self._dt.from_host(data)
        if is_physical:
            self.setp(data)
            self.to_spectral()
        else:
            data = as_device(data, torch.complex128, self._device)
            if tuple(data.shape) != tuple(self._sdata.shape):
                data = scale_variable(data, self._params)
            self.sets(data)

    def pddx(self):
        return self._sd.pddx(self.getp())

    def pddz(self):
        return self._sd.pddz(self.getp())

    def sddx(self):
        return self._sd.sddx(self.gets(), self._basis_functions[0])

    def sddz(self):
        return self._sd.sddz(self.gets(), self._basis_functions[1])

    def sd2dx2(self):
        return self._sd.sd2dx2(self.gets(), self._basis_functions[0])

    def sd2dz2(self):
        return self._sd.sd2dz2(self.gets(), self._basis_functions[1])

    def snabla2(self):
        """sd2dx2 + sd2dz2 (melvin/Variable.py:111-113), one kernel."""
        return self._sd.snabla2(self.gets(), tuple(self._basis_functions))

    def lap(self):
        return self._sd.calc_lap(self._basis_functions)

    def vec_dot_nabla(self, ux, uz, out=None, convert_to_physical=True):
        """``to_spectral(pddx(ux q) + pddz(uz q))`` (melvin/Variable.py:119-128).

        The physical form of this variable is refreshed as a side effect, as
        in the reference.  With ``convert_to_physical=False`` the current
        physical data is used as is.
        """
        st = self._st
        pl = st._plan
        dev = self._device
        uxd = as_device(ux, torch.float64, dev, pl.physical_shape)
        uzd = as_device(uz, torch.float64, dev, pl.physical_shape)
        res = torch.empty(pl.spectral_shape, dtype=torch.complex128, device=dev)
        if convert_to_physical and out is None:
            pl.call("mgb_vec_dot_nabla", N.ptr(self._sdata), N.ptr(self._pdata), N.ptr(uxd), N.ptr(uzd),
                    N.ptr(res), N.ptr(pl.work()), N.stream_handle(dev))
            return res
        # explicit form: the physical J is also left in `out`
        if convert_to_physical:
            self.to_physical()
        j = self._sd.pddx(uxd * self._pdata) + self._sd.pddz(uzd * self._pdata)
        if out is not None:
            out[...] = j if isinstance(out, torch.Tensor) else j.cpu().numpy()
        st.to_spectral(j, res, self._basis_functions)
        return res

    def save(self, dump_counter):
        fname = self._dump_name + f"{dump_counter:04d}.npy"
        np.save(fname, self._pdata.cpu().numpy())

    def on_host(self):
        return self._sdata.cpu().numpy()

    def get_name(self):
        return self._dump_name


def scale_variable(var, params):
    """Resample a spectral array to this grid's spectral shape, keeping the
    overlapping low modes (the intent of melvin/Variable.py:142-151, which
    targets the fully spectral ``(2nn+1, nm)`` layout; complex values are
    kept)."""
    rows, cols = params.spectral_shape
    out = torch.zeros((rows, cols), dtype=torch.complex128, device=var.device)
    if params.is_fully_spectral():
        nn_in = (var.shape[0] - 1) // 2
        k = min(nn_in, params.nn)
        c = min(var.shape[1], cols)
        out[: k + 1, :c] = var[: k + 1, :c]
        if k > 0:
            out[-k:, :c] = var[-k:, :c]
    else:
        r = min(var.shape[0], rows)
        c = min(var.shape[1], cols)
        out[:r, :c] = var[:r, :c]
    return out
