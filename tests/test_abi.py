"""The C ABI without a GPU: the library loads, exports every function
include/melvin_gb300.h declares, and the ctypes structures have the C
layout (checked against a program compiled from the header)."""

import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "melvin_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:int|const char\*)\s+(mgb_\w+)\(", text, re.M)))


def test_header_declares_the_entry_points():
    names = declared_functions()
    for must in ("mgb_plan_create", "mgb_to_physical", "mgb_vec_dot_nabla", "mgb_step", "mgb_step_prepare",
                 "mgb_poisson_solve", "mgb_integrate_semi_implicit", "mgb_diagnostics"):
        assert must in names


def test_library_exports_every_declared_symbol():
    from melvin import _native

    if not _native.LIB_PATH.exists():
        pytest.skip("library not built (run __graft_entry__.build())")
    lib = C.CDLL(str(_native.LIB_PATH))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    # every declared symbol has a ctypes signature in the binding
    assert set(declared_functions()) <= set(_native.SIGNATURES)


def test_status_strings_without_gpu():
    from melvin import _native

    if not _native.LIB_PATH.exists():
        pytest.skip("library not built")
    lib = _native.load_library()
    assert lib.mgb_status_string(0) == b"ok"
    assert lib.mgb_status_string(2) == b"unsupported configuration"
    # argument validation happens before any CUDA call
    assert lib.mgb_plan_create(None, None) == _native.MGB_ERR_INVALID
    assert b"null pointer" in lib.mgb_last_error()


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_ctypes_struct_layout_matches_c(tmp_path):
    from melvin import _native as N

    src = tmp_path / "layout.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "melvin_gb300.h"\n'
        "int main(void){\n"
        'printf("%zu %zu %zu %zu\\n", sizeof(mgb_grid), sizeof(mgb_term), sizeof(mgb_field_eq), sizeof(mgb_equation));\n'
        'printf("%zu %zu %zu %zu\\n", offsetof(mgb_grid, lx), offsetof(mgb_grid, precision),'
        " offsetof(mgb_field_eq, terms), offsetof(mgb_equation, f));\n"
        'printf("%zu %zu %zu %zu %zu\\n", sizeof(mgb_batch), offsetof(mgb_batch, members),'
        " offsetof(mgb_batch, term_coef), sizeof(mgb_tile_info), offsetof(mgb_tile_info, smem_bytes));\n"
        'printf("%zu %zu %zu %zu %zu\\n", sizeof(mgb_run_state), offsetof(mgb_run_state, status),'
        " offsetof(mgb_run_state, diag), sizeof(mgb_run_config), offsetof(mgb_run_config, tracker_ke));\n"
        'printf("%zu %zu\\n", offsetof(mgb_equation, diag_flux), offsetof(mgb_run_config, tracker_flux));\n'
        "return 0;}\n"
    )
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    sizes = list(map(int, out[:4]))
    offs = list(map(int, out[4:8]))
    more = list(map(int, out[8:13]))
    run = list(map(int, out[13:18]))
    tail = list(map(int, out[18:]))
    assert sizes == [C.sizeof(N.MgbGrid), C.sizeof(N.MgbTerm), C.sizeof(N.MgbFieldEq), C.sizeof(N.MgbEquation)]
    assert offs == [N.MgbGrid.lx.offset, N.MgbGrid.precision.offset, N.MgbFieldEq.terms.offset,
                    N.MgbEquation.f.offset]
    assert more == [C.sizeof(N.MgbBatch), N.MgbBatch.members.offset, N.MgbBatch.term_coef.offset,
                    C.sizeof(N.MgbTileInfo), N.MgbTileInfo.smem_bytes.offset]
    assert run == [C.sizeof(N.MgbRunState), N.MgbRunState.status.offset, N.MgbRunState.diag.offset,
                   C.sizeof(N.MgbRunConfig), N.MgbRunConfig.tracker_ke.offset]
    assert tail == [N.MgbEquation.diag_flux.offset, N.MgbRunConfig.tracker_flux.offset]
