"""GB300 (sm_103a) implementation of Melvin.py's per-timestep hot path.

Drop-in for the reference package ``melvin``: the same classes and
functions, with every array a CUDA tensor and every numerical verb a
hand-written kernel of ``libmelvin_gb300.so`` (C ABI in
include/melvin_gb300.h).  :mod:`melvin.stepper` adds a fused timestep.
"""

from .ArrayFactory import ArrayFactory
from .BasisFunctions import BasisFunctions
from .DataTransferer import DataTransferer
from .Integrator import Integrator
from .utility import load_scipy_sparse, load_scipy_sparse_linalg
from .LaplacianSolver import LaplacianSolver
from .Parameters import Parameters
from .ScalarTracker import ScalarTracker
from .SpatialDifferentiator import SpatialDifferentiator
from .SpectralTransformer import SpectralTransformer
from .Ticker import Ticker
from .TimeDerivative import TimeDerivative
from .Timer import Timer
from .Variable import Variable
from .Simulation import Simulation
from .stepper import FieldEquation, Stepper, Term
from . import autotune, equations

__all__ = [
    "ArrayFactory", "BasisFunctions", "DataTransferer", "Integrator", "LaplacianSolver", "Parameters",
    "ScalarTracker", "SpatialDifferentiator", "SpectralTransformer", "Ticker", "TimeDerivative", "Timer",
    "Variable", "Simulation", "FieldEquation", "Stepper", "Term", "autotune", "equations",
    "load_scipy_sparse", "load_scipy_sparse_linalg",
]
