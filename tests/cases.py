"""Grid and problem definitions shared by the tests (the same cases the
golden vectors were generated for)."""

import numpy as np

import oracle as O
from oracle import problems as P

TWO_PI = 2 * np.pi

# tag -> (nx, nz, lx, lz, fdm_z, order, integrator_order, integrator)
VERB_CASES = {
    "fs32_o2": (32, 32, TWO_PI, TWO_PI, False, 2, 2, "semi-implicit"),
    "fs32x64_o4": (32, 64, 1.0, 2.0, False, 4, 4, "semi-implicit"),
    "fd32x17_o2": (32, 17, 2.0, 1.0, True, 2, 2, "explicit"),
    "fd64x21_o4": (64, 21, 2.0, 1.0, True, 4, 4, "explicit"),
}

# tag -> (grid, specs, field names, integrator, order, dt)
TRAJ_CASES = {
    "tg32_o2_ab2": (O.Grid(32, 32, TWO_PI, TWO_PI, False, 2), P.vorticity_specs(1e-2), ["w"], "semi-implicit", 2, 1e-2),
    "tg32_o4_ab4": (O.Grid(32, 32, TWO_PI, TWO_PI, False, 4), P.vorticity_specs(1e-2), ["w"], "semi-implicit", 4, 1e-2),
    "kh64x32": (O.Grid(64, 32, TWO_PI, TWO_PI, False, 2), P.kh_specs(1e-3, 2e-3), ["w", "c"], "semi-implicit", 2, 5e-3),
    "ddcs32": (O.Grid(32, 32, 4.0, 2.0, False, 2), P.ddc_spectral_specs(7.0, 1.1, 1.0 / 3.0), ["w", "tmp", "xi"],
               "semi-implicit", 2, 1e-3),
    "rbc32x17_o4_ab4": (O.Grid(32, 17, 2.0, 1.0, True, 4), P.rbc_specs(1.0, 1e5), ["w", "tmp"], "explicit", 4, 1e-5),
    "rbc32x17_o2_ab2": (O.Grid(32, 17, 2.0, 1.0, True, 2), P.rbc_specs(1.0, 1e5), ["w", "tmp"], "explicit", 2, 1e-5),
    "rbc32x17_pece4": (O.Grid(32, 17, 2.0, 1.0, True, 4), P.rbc_specs(1.0, 1e5), ["w", "tmp"], "pece", 4, 1e-5),
    "ddcd32x17": (O.Grid(32, 17, 2.0, 1.0, True, 2), P.ddc_dirichlet_specs(7.0, 1e5, 2.0, 10.0), ["w", "T", "S"],
                  "explicit", 2, 2e-6),
}


def grid_of(tag):
    nx, nz, lx, lz, fdm, order, _, _ = VERB_CASES[tag]
    return O.Grid(nx, nz, lx, lz, fdm, order)


def params_dict(g, integrator="semi-implicit", order=2, dt=1e-3, precision="double", device="cuda:0"):
    return {
        "nx": g.nx, "nz": g.nz, "lx": g.lx, "lz": g.lz, "final_time": 1.0, "initial_dt": dt,
        "spatial_derivative_order": g.order, "integrator_order": order, "integrator": integrator,
        "discretisation": ["spectral", "fdm" if g.fdm_z else "spectral"], "precision": precision,
        "device": device,
    }


# Cosine / sine basis golden cases: tag -> grid (n = 2^k + 1 on a mirrored axis),
# basis codes in the tag suffix (0 complex exponential, 1 cosine, 2 sine).
BASIS_TAGS = ["basis65x64_10", "basis65x64_20", "basis64x65_01", "basis64x65_02", "basis65x65_11", "basis65x65_22",
              "basis65x65_21", "basis33x65_12",
              # transform lengths that are not powers of two: 78 x 48, 48 x 78, 64 x 88, 24 x 36, 258 x 198
              "basis40x48_10", "basis48x40_02", "basis33x45_21", "basis24x36_00", "basis130x100_11"]


def basis_grid(tag):
    nx, nz = (int(v) for v in tag[len("basis"):].split("_")[0].split("x"))
    return O.Grid(nx, nz, 1.0, 2.0)

# Integrator.set_dt golden cases: tag -> grid
CFL_GRIDS = {
    "cfl_fs32": O.Grid(32, 32, TWO_PI, TWO_PI),
    "cfl_fd32x17": O.Grid(32, 17, 2.0, 1.0, True, 2),
}
CFL_E2E_GRIDS = {
    "cfl_e2e_fs32": O.Grid(32, 32, TWO_PI, TWO_PI),
    "cfl_e2e_fd32x17": O.Grid(32, 17, 2.0, 1.0, True, 2),
}
CFL_CUTOFF = 0.5  # Parameters.cfl_cutoff default (melvin/Parameters.py:14)
