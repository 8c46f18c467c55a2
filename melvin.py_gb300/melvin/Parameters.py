"""Run parameters (melvin/Parameters.py of the reference).

Same keys, defaults, validation and derived-shape rules as the reference
(melvin/Parameters.py:6-96).  Extra keys understood here:

* ``precision = "split"``: FP32 transforms, derivatives and products with an
  FP64 spectral state and history (``"single"`` is treated the same way, so
  state stays complex128 in every mode);
* ``precision = "dfloat"``: transforms, derivatives and products in
  double-float arithmetic (pairs of FP32 numbers, 48-bit significand) on the
  FP32 pipes, with an FP64 state and history -- FP64-class accuracy at a
  fraction of the cost of FP64 arithmetic on GB300;
* ``device``: the CUDA device that holds every array (default ``"cuda"``).
"""

import json
import sys

import numpy as np


class Parameters:
    required_params = ["nx", "nz", "lx", "lz", "final_time"]

    # defaults (melvin/Parameters.py:9-30)
    integrator_order = 2
    integrator = "semi-implicit"
    spatial_derivative_order = 2
    alpha = 0.51
    cfl_cutoff = 0.5
    cfl_cadence = 10
    tracker_cadence = 100
    save_cadence = 100
    load_from = None
    discretisation = ["spectral", "spectral"]
    precision = "double"
    device = "cuda"

    nx = None
    nz = None
    lx = None
    lz = None
    final_time = None

    def __init__(self, params, validate=True):
        if validate and not self.is_valid(params):
            sys.exit(-1)
        self.load_from_dict(params)
        self._original_params = params

    def load_from_dict(self, params):
        for key, value in params.items():
            setattr(self, key, value)
        self.set_derived_params(params)

    def is_valid(self, params):
        ok = True
        for key in self.required_params:
            if key not in params:
                print(key, "missing from input parameters.")
                ok = False
        return int(ok)

    def is_fully_spectral(self):
        return self.discretisation[0] == "spectral" and self.discretisation[1] == "spectral"

    def set_derived_params(self, params):
        """melvin/Parameters.py:63-92."""
        if "dump_cadence" not in params:
            self.dump_cadence = 0.1 * self.final_time
        if self.discretisation[0] == "spectral":
            self.nn = (self.nx - 1) // 3
        if self.discretisation[1] == "spectral":
            self.nm = (self.nz - 1) // 3
        if self.is_fully_spectral():
            self.spectral_shape = (2 * self.nn + 1, self.nm)
        elif self.discretisation[0] == "fdm":
            self.spectral_shape = (self.nx, self.nm)
        elif self.discretisation[1] == "fdm":
            self.spectral_shape = (self.nn, self.nz)
        self.physical_shape = (self.nx, self.nz)
        self.dx = self.lx / self.nx
        self.dz = self.lz / self.nz
        if self.precision in ("double", "split", "single", "dfloat"):
            # the prognostic state is FP64 in every precision mode
            self.complex = np.complex128
            self.float = np.float64
        else:
            raise ValueError(f"precision={self.precision!r}: use 'double', 'dfloat', 'split' or 'single'")
        if "initial_dt" not in params:
            self.initial_dt = 0.2 * min(self.dx, self.dz)

    def save(self, fname="params.json"):
        with open(fname, "w") as fp:
            json.dump(self._original_params, fp)
