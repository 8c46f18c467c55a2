"""ctypes binding of ``libmelvin_gb300.so`` (the C ABI in include/melvin_gb300.h).

The library is the only compute path: when it is missing, or no CUDA device
is visible, creating a plan raises instead of falling back to the CPU.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

import torch

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libmelvin_gb300.so"

MGB_OK = 0
MGB_ERR_INVALID = 1
MGB_ERR_UNSUPPORTED = 2
MGB_ERR_CUDA = 3
MGB_ERR_NONFINITE = 4
MGB_ERR_CFL = 5
MGB_ERR_NOMEM = 6

PREC_DOUBLE = 0
PREC_SPLIT = 1
PREC_DFLOAT = 2
PRECISIONS = {"double": PREC_DOUBLE, "split": PREC_SPLIT, "single": PREC_SPLIT, "dfloat": PREC_DFLOAT}

INT_SEMI_IMPLICIT = 0
INT_EXPLICIT = 1
INT_PECE = 2

BC_ZERO_M0 = 1
BC_DIRICHLET_W = 2
BC_DIRICHLET_T = 4

DDX, DDZ, D2DX2, D2DZ2, NABLA2 = range(5)


class MelvinError(RuntimeError):
    """A native call returned an error status."""

    def __init__(self, status, message):
        super().__init__(f"{message} [status {status}]")
        self.status = status


class MelvinUnsupported(MelvinError, NotImplementedError):
    pass


class MelvinInvalid(MelvinError, ValueError):
    pass


class MgbGrid(C.Structure):
    _fields_ = [
        ("nx", C.c_int32),
        ("nz", C.c_int32),
        ("lx", C.c_double),
        ("lz", C.c_double),
        ("fdm_z", C.c_int32),
        ("sdo", C.c_int32),
        ("precision", C.c_int32),
    ]


class MgbTerm(C.Structure):
    _fields_ = [("src", C.c_int32), ("op", C.c_int32), ("coef", C.c_double)]


class MgbFieldEq(C.Structure):
    _fields_ = [
        ("kappa", C.c_double),
        ("nterms", C.c_int32),
        ("terms", MgbTerm * 4),
        ("bc", C.c_int32),
    ]


class MgbBatch(C.Structure):
    _fields_ = [
        ("count", C.c_int32),
        ("members", C.c_void_p),
        ("q", C.c_void_p),
        ("hist", C.c_void_p),
        ("term_coef", C.c_void_p),
    ]


class MgbTileInfo(C.Structure):
    _fields_ = [
        ("available", C.c_int32),
        ("shape", C.c_int32),
        ("radix", C.c_int32),
        ("kind", C.c_int32),
        ("smem_bytes", C.c_uint64),
    ]


class MgbRunState(C.Structure):
    _fields_ = [
        ("t", C.c_double),
        ("dt", C.c_double),
        ("loop", C.c_int64),
        ("stop_loop", C.c_int64),
        ("cfl_counter", C.c_int64),
        ("tracker_counter", C.c_int64),
        ("cfl_fired", C.c_int64),
        ("tracker_fired", C.c_int64),
        ("status", C.c_int32),
        ("dt_changed", C.c_int32),
        ("ntracked", C.c_int32),
        ("dropped", C.c_int32),
        ("diag", C.c_double * 4),
    ]


class MgbRunConfig(C.Structure):
    _fields_ = [
        ("final_time", C.c_double),
        ("cfl_cutoff", C.c_double),
        ("cfl_cadence", C.c_int32),
        ("tracker_cadence", C.c_int32),
        ("capacity", C.c_int32),
        ("horizon", C.c_int32),
        ("pause_time", C.c_double),
        ("tracker_t", C.c_void_p),
        ("tracker_ke", C.c_void_p),
        ("tracker_flux", C.c_void_p),
    ]


RUN_RUNNING, RUN_FINISHED, RUN_CFL_BREACH, RUN_PAUSED = 0, 1, 2, 3
RUN_TICK, RUN_CFL, RUN_TRACK = 1, 2, 4

# kernel families of the fused step with tile variants (mgb_family)
FAMILY_XINV, FAMILY_ZSTEP, FAMILY_XFWD = 0, 1, 2
FAMILIES = ("xinv", "zstep", "xfwd")
TILE_VARIANTS = 5


class MgbEquation(C.Structure):
    _fields_ = [
        ("nfields", C.c_int32),
        ("integrator", C.c_int32),
        ("order", C.c_int32),
        ("alpha", C.c_double),
        ("f", MgbFieldEq * 3),
        ("diag_flux", C.c_int32),
    ]


_P = C.c_void_p
_I = C.c_int32
_D = C.c_double

# name -> argtypes (all return int32 status unless listed in _RESTYPES)
SIGNATURES = {
    "mgb_plan_create": [C.POINTER(MgbGrid), C.POINTER(_P)],
    "mgb_plan_destroy": [_P],
    "mgb_plan_shapes": [_P, C.POINTER(_I), C.POINTER(_I), C.POINTER(_I), C.POINTER(_I)],
    "mgb_workspace_bytes": [_P, _I, _I, C.POINTER(C.c_size_t)],
    "mgb_status_string": [_I],
    "mgb_last_error": [],
    "mgb_to_physical": [_P, _P, _P, _P, _P],
    "mgb_to_spectral": [_P, _P, _P, _P, _P],
    "mgb_to_physical_basis": [_P, _I, _I, _P, _P, _P, _P],
    "mgb_to_spectral_basis": [_P, _I, _I, _P, _P, _P, _P],
    "mgb_spectral_derivative_basis": [_P, _I, _I, _I, _P, _P, _P],
    "mgb_laplacian_basis": [_P, _I, _I, _P, _P],
    "mgb_poisson_solve_basis": [_P, _I, _I, _P, _P, _P],
    "mgb_pddx": [_P, _P, _P, _P],
    "mgb_pddz": [_P, _P, _P, _P],
    "mgb_spectral_derivative": [_P, _I, _P, _P, _P],
    "mgb_laplacian": [_P, _P, _P],
    "mgb_poisson_solve": [_P, _P, _P, _P],
    "mgb_vec_dot_nabla": [_P, _P, _P, _P, _P, _P, _P, _P],
    "mgb_vec_dot_nabla_noalloc": [_P, _P, _P, _P, _P, _P, _P],
    "mgb_velocity_from_vorticity": [_P, _P, _P, _P, _P, _P, _P, _P, _P, _P],
    "mgb_integrate_semi_implicit": [_P, _P, _P, _I, _I, _D, _D, _P, _P],
    "mgb_integrate_explicit": [_P, _P, _P, _I, _I, _D, _P, _P],
    "mgb_adams": [_P, _I, _P, _I, _I, _D, _P, _P],
    "mgb_diagnostics": [_P, _P, _P, _P, _P, _P],
    "mgb_step": [_P, C.POINTER(MgbEquation), C.POINTER(_P), C.POINTER(_P), _I, _D, _P, _P, _P],
    "mgb_step_prepare": [_P, C.POINTER(MgbEquation), _D, _P, _P],
    "mgb_batch_workspace_bytes": [_P, _I, _I, C.POINTER(C.c_size_t)],
    "mgb_batch_step": [_P, C.POINTER(MgbEquation), C.POINTER(MgbBatch), _I, _D, _P, _P, _P],
    "mgb_step_kernel_count": [_P, C.POINTER(MgbEquation), C.POINTER(_I)],
    "mgb_step_events": [_P, C.POINTER(MgbEquation), C.POINTER(_P), C.POINTER(_P), _I, _D, _P, _P, _P,
                        C.POINTER(_P), _I],
    "mgb_step_waits": [_P, C.POINTER(MgbEquation), C.POINTER(_P), C.POINTER(_P), _I, _D, _P, _P, _P,
                       C.POINTER(_P), _I],
    "mgb_run_begin": [_P, _P, C.POINTER(MgbRunConfig), _P],
    "mgb_run_step": [_P, C.POINTER(MgbEquation), C.POINTER(_P), C.POINTER(_P), _I, C.c_int64, _I, _P, _P,
                     C.POINTER(MgbRunConfig), _P],
    "mgb_tile_info_get": [_P, _I, _I, _I, C.POINTER(MgbTileInfo)],
    "mgb_plan_set_tiles": [_P, _I, C.POINTER(_I)],
    "mgb_plan_get_tiles": [_P, _I, C.POINTER(_I)],
    "mgb_fp64_fma_probe": [_P, _I, _I, C.POINTER(_D), _P],
}
_RESTYPES = {"mgb_status_string": C.c_char_p, "mgb_last_error": C.c_char_p}

_lib = None
_lib_lock = threading.Lock()


def load_library(path: Path | None = None):
    """Load (once) and return the native library, declaring every signature."""
    global _lib
    with _lib_lock:
        if _lib is not None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise ImportError(
                f"native library {p} is missing; build it with __graft_entry__.build() "
                "or `python -m melvin._build` (there is no CPU fallback)"
            )
        lib = C.CDLL(str(p))
        for name, args in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = _RESTYPES.get(name, C.c_int32)
        _lib = lib
        return lib


def check(status: int):
    if status == MGB_OK:
        return
    lib = load_library()
    msg = lib.mgb_last_error().decode(errors="replace") or lib.mgb_status_string(status).decode()
    if status == MGB_ERR_UNSUPPORTED:
        raise MelvinUnsupported(status, msg)
    if status == MGB_ERR_INVALID:
        raise MelvinInvalid(status, msg)
    if status == MGB_ERR_CFL:
        raise RuntimeError("CFL condition breached")
    raise MelvinError(status, msg)


def ptr(t: torch.Tensor | None):
    return None if t is None else C.c_void_p(t.data_ptr())


def stream_handle(device=None):
    return C.c_void_p(torch.cuda.current_stream(device).cuda_stream)


class Plan:
    """A native plan: grid constants, twiddle tables, Dirichlet factors and
    the per-verb scratch buffer (allocated once with torch)."""

    def __init__(self, nx, nz, lx, lz, fdm_z, sdo, precision, device):
        if not torch.cuda.is_available():
            raise RuntimeError("melvin GB300 kernels need a CUDA device; none is visible (no CPU fallback)")
        self.lib = load_library()
        self.device = torch.device(device)
        g = MgbGrid(int(nx), int(nz), float(lx), float(lz), int(bool(fdm_z)), int(sdo), int(precision))
        self.grid = g
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            check(self.lib.mgb_plan_create(C.byref(g), C.byref(h)))
        self.handle = h
        r, c, pr, pc = _I(), _I(), _I(), _I()
        check(self.lib.mgb_plan_shapes(h, C.byref(r), C.byref(c), C.byref(pr), C.byref(pc)))
        self.spectral_shape = (r.value, c.value)
        self.physical_shape = (pr.value, pc.value)
        self._work = None
        self._step_work = {}
        self.last_prepared = None  # the Stepper whose coefficients the plan last prepared

    def workspace_bytes(self, family, nfields=1):
        b = C.c_size_t()
        check(self.lib.mgb_workspace_bytes(self.handle, family, nfields, C.byref(b)))
        return b.value

    def work(self):
        if self._work is None:
            n = self.workspace_bytes(0)
            self._work = torch.empty(n, dtype=torch.uint8, device=self.device)
        return self._work

    def step_work(self, nfields):
        w = self._step_work.get(nfields)
        if w is None:
            n = self.workspace_bytes(1, nfields)
            w = torch.empty(n, dtype=torch.uint8, device=self.device)
            self._step_work[nfields] = w
        return w

    def call(self, name, *args):
        check(getattr(self.lib, name)(self.handle, *args))

    # ---- tile variants of the fused step (fully spectral plans) ----------

    def tile_info(self, family, nfields, variant):
        """(available, shape, radix, smem_bytes, kind) of one tile variant
        (kind 0: shared-memory passes, 1: register-resident points)."""
        info = MgbTileInfo()
        self.call("mgb_tile_info_get", int(family), int(nfields), int(variant), C.byref(info))
        return bool(info.available), info.shape, info.radix, info.smem_bytes, info.kind

    def get_tiles(self, nfields):
        t = (_I * 3)()
        self.call("mgb_plan_get_tiles", int(nfields), t)
        return tuple(t)

    def set_tiles(self, nfields, tiles):
        t = (_I * 3)(*[int(v) for v in tiles])
        self.call("mgb_plan_set_tiles", int(nfields), t)

    def __del__(self):
        try:
            if getattr(self, "handle", None) and self.handle.value and _lib is not None:
                _lib.mgb_plan_destroy(self.handle)
        except Exception:
            pass


_plans = {}


def plan_for(params, device=None) -> Plan:
    """Cached plan of a Parameters object (one per grid, precision, device)."""
    dev = torch.device(device if device is not None else getattr(params, "device", "cuda"))
    if dev.type == "cuda" and dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    fdm = params.discretisation[1] == "fdm"
    if params.discretisation[0] != "spectral":
        raise NotImplementedError("Finite difference not implemented in x direction")
    prec = PRECISIONS[params.precision]
    key = (params.nx, params.nz, float(params.lx), float(params.lz), fdm, params.spatial_derivative_order, prec, str(dev))
    p = _plans.get(key)
    if p is None:
        p = Plan(params.nx, params.nz, params.lx, params.lz, fdm, params.spatial_derivative_order, prec, dev)
        _plans[key] = p
    return p
