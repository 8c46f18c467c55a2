"""Basis-function enum and derivative factors (melvin/BasisFunctions.py).

The enum values and the factor rules are part of the reference's API: first
derivative factor ``2*pi*i/L`` for complex exponentials, ``+-pi/L`` for
sine/cosine, 0 for FDM; second derivative ``-|factor|^2``.  Only
COMPLEX_EXP (x and z) and FDM (z) are computed on the GPU.
"""

from enum import IntEnum

import numpy as np


class BasisFunctions(IntEnum):
    COMPLEX_EXP = 0
    COSINE = 1
    SINE = 2
    FDM = 3


def is_spectral(bs):
    return bs in (BasisFunctions.COMPLEX_EXP, BasisFunctions.COSINE, BasisFunctions.SINE)


def is_fully_spectral(bs1, bs2):
    return is_spectral(bs1) and is_spectral(bs2)


def calc_diff_wavelength(basis_fn):
    if basis_fn is BasisFunctions.COMPLEX_EXP:
        return 1j * 2 * np.pi
    if basis_fn is BasisFunctions.SINE:
        return np.pi
    if basis_fn is BasisFunctions.COSINE:
        return -np.pi
    return 0


def calc_diff2_wavelength(basis_fn):
    return -np.abs(calc_diff_wavelength(basis_fn)) ** 2


def calc_diff_factor(basis_fn, length):
    return calc_diff_wavelength(basis_fn) / length


def gen_diff_factors(length):
    return [calc_diff_wavelength(b) / length for b in BasisFunctions]


def gen_diff2_factors(length):
    return [calc_diff2_wavelength(b) / length ** 2 for b in BasisFunctions]
