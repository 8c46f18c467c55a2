"""Simulation driver (melvin/Simulation.py): owns the numerics objects, the
loop clock and the tickers.

Differences from the reference, all at the host level:
* ``dump``/``load`` write and read a pickle-free ``.npz`` (params as JSON,
  ticker state as flat keys), so ``load`` works (the reference's load fails
  on its own pickled entries);
* ``make_stepper`` builds a fused timestep (see :mod:`melvin.stepper`).
"""

import json

import numpy as np

from .ArrayFactory import ArrayFactory
from .DataTransferer import DataTransferer
from .Integrator import Integrator
from .LaplacianSolver import LaplacianSolver
from .ScalarTracker import ScalarTracker
from .SpatialDifferentiator import SpatialDifferentiator
from .SpectralTransformer import SpectralTransformer
from .stepper import Stepper
from .Ticker import Ticker
from .TimeDerivative import TimeDerivative
from .Timer import Timer
from .Variable import Variable


class Simulation:
    def __init__(self, params, xp=None):
        self._params = params
        self._xp = xp
        self._data_trans = DataTransferer(xp, getattr(params, "device", "cuda"))
        self._integrator = Integrator(params, xp)
        self._array_factory = ArrayFactory(params, xp)
        self._spatial_diff = SpatialDifferentiator(params, xp, self._array_factory)
        self._spectral_trans = SpectralTransformer(params, xp, self._array_factory)
        self._t = 0
        self._loop_counter = 0
        self._dump_vars = []
        self._dump_dvars = []
        self._dump_idx = 0
        self._save_vars = []
        self._tickers = []
        self._timer = Timer()
        self._wallclock_remaining = 0.0
        self._wallclock_ticker = Ticker(100, self.calc_time_remaining, is_loop_counter=True)
        self.register_ticker(self._wallclock_ticker)

    def make_variable(self, name, basis_fns):
        return Variable(self._params, self._xp, sd=self._spatial_diff, st=self._spectral_trans,
                        dt=self._data_trans, array_factory=self._array_factory, dump_name=name,
                        basis_functions=basis_fns)

    def make_derivative(self, name):
        return TimeDerivative(self._params, self._xp, dump_name=name)

    def init_laplacian_solver(self, basis_fns):
        self._laplacian_solver = LaplacianSolver(self._params, self._xp, basis_fns,
                                                 spatial_diff=self._spatial_diff,
                                                 array_factory=self._array_factory)

    def make_stepper(self, fields, **kw):
        return Stepper(self, fields, **kw)

    def config_dump(self, variables, derivatives):
        self._dump_vars = variables
        self._dump_dvars = derivatives
        self._dump_ticker = Ticker(self._params.dump_cadence, self.dump, dump_name="dump_ticker",
                                   is_loop_counter=False)
        self.register_ticker(self._dump_ticker)

    def config_save(self, variables):
        self._save_vars = variables
        self._save_ticker = Ticker(self._params.save_cadence, self.save, dump_name="save_ticker",
                                   is_loop_counter=False)
        self.register_ticker(self._save_ticker)

    def config_cfl(self, ux, uz):
        self._ux = ux
        self._uz = uz
        self._cfl_ticker = Ticker(self._params.cfl_cadence, self.set_dt, dump_name="cfl_ticker",
                                  is_loop_counter=True)
        self.register_ticker(self._cfl_ticker)

    def config_scalar_trackers(self, trackers):
        self._tracker_fns = [trackers[k] for k in trackers]
        self._trackers = [ScalarTracker(self._params, self._xp, k) for k in trackers]
        self._tracker_ticker = Ticker(self._params.tracker_cadence, self.track_scalars,
                                      dump_name="tracker_ticker", is_loop_counter=True)
        self.register_ticker(self._tracker_ticker)
        self._save_vars += self._trackers

    def track_scalars(self, ticker):
        for tracker, fn in zip(self._trackers, self._tracker_fns):
            tracker.append(self._t, fn())

    def set_dt(self, ticker):
        self._integrator.set_dt(self._ux, self._uz)

    def save(self, ticker):
        self.print_info()
        for var in self._save_vars:
            var.save(ticker.times_fired)

    def print_info(self):
        hours = int(self._wallclock_remaining / 3600)
        minutes = int((self._wallclock_remaining / 3600.0 - hours) * 60)
        print(f"{self._t / self._params.final_time * 100:.2f}% complete", f"t = {self._t:.2e}",
              f"dt = {self._integrator._dt:.2e}", f"Remaining: {hours} hr, {minutes} min")

    def form_dumpname(self, index):
        return f"dump{index:04d}.npz"

    def dump(self, ticker):
        fname = self.form_dumpname(ticker.times_fired)
        data = {v.get_name(): self._data_trans.to_host(v[:]) for v in self._dump_vars}
        data.update({d.get_name(): self._data_trans.to_host(d.get_all()) for d in self._dump_dvars})
        for tk in self._tickers:
            st = tk.dump()
            data[f"{tk.get_name()}.counter"] = np.float64(st["counter"])
            data[f"{tk.get_name()}.times_fired"] = np.int64(st["times_fired"])
        np.savez(fname, **data,
                 curr_idx=np.int64(self._dump_dvars[0].get_curr_idx() if self._dump_dvars else 0),
                 dt=np.float64(self._integrator._dt), t=np.float64(self._t),
                 loop_counter=np.int64(self._loop_counter),
                 params=np.array(json.dumps(self._params._original_params, default=str)))

    def load(self, index):
        fname = self.form_dumpname(index)
        with np.load(fname, allow_pickle=False) as d:
            for v in self._dump_vars:
                v.load(d[v._dump_name])
            for dv in self._dump_dvars:
                dv.load(d[dv._dump_name])
                dv.set_curr_idx(int(d["curr_idx"]))
            for tk in self._tickers:
                key = tk._dump_name
                if f"{key}.counter" in d:
                    tk.restore({"counter": float(d[f"{key}.counter"]),
                                "times_fired": int(d[f"{key}.times_fired"])})
            self._integrator._dt = float(d["dt"])
            self._t = float(d["t"])
            self._loop_counter = int(d["loop_counter"])

    def is_running(self):
        return self._t < self._params.final_time

    def register_ticker(self, ticker):
        self._tickers.append(ticker)

    def end_loop(self):
        self._loop_counter += 1
        self._t += self._integrator._dt
        for ticker in self._tickers:
            ticker.tick(self._t, self._loop_counter)

    def calc_time_remaining(self, ticker):
        self._timer.split()
        per_step = self._timer.diff / ticker._cadence
        self._wallclock_remaining = per_step * (self._params.final_time - self._t) / self._integrator._dt

    def get_laplacian_solver(self):
        return self._laplacian_solver
