"""CPU oracle for the Melvin.py per-timestep hot path.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (the ``melvin`` package under
``melvin.py_gb300/`` and its CUDA library) imports, links or runs this
package.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` (``cpu_baseline`` and ``--impl reference``) use it, and only as
the thing that is checked against or timed beside the GPU path.

The oracle is a NumPy/SciPy restatement of the reference algorithm.  Every
function cites the reference file and lines (paths relative to the Melvin.py
project root) whose behaviour it restates.  It is pinned against golden
vectors produced by running the reference itself (``tests/golden/``), see
``tests/test_oracle_golden.py``.
"""

from .melvin_np import (  # noqa: F401
    Grid,
    mode_numbers,
    to_physical,
    to_spectral,
    pddx,
    pddz,
    pd2dz2,
    sddx,
    sddz,
    sd2dx2,
    sd2dz2,
    snabla2,
    laplacian_symbol,
    PoissonSolver,
    vec_dot_nabla,
    velocity_from_vorticity,
    History,
    adams_bashforth,
    adams_moulton,
    semi_implicit_update,
    explicit_update,
    kinetic_energy,
    cfl_dt,
)
from . import problems  # noqa: F401
