"""Build step for the native library ``libmelvin_gb300.so``.

Compiles every ``csrc/*.cu`` translation unit for sm_103a with nvcc, in
parallel, and links them (static CUDA runtime) into
``melvin/_lib/libmelvin_gb300.so``.  Objects go to ``melvin.py_gb300/_build``.
An object is rebuilt when it is older than its source or any header.

Run directly (``python -m melvin._build`` from ``melvin.py_gb300``) or via
``__graft_entry__.build()`` at the repository root.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent            # melvin.py_gb300/melvin
ROOT = PKG_DIR.parent                                 # melvin.py_gb300
CSRC = ROOT / "csrc"
INCLUDE = ROOT.parent / "include"
BUILD = ROOT / "_build"
LIB_DIR = PKG_DIR / "_lib"
LIB_NAME = "libmelvin_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off keeps host-side table arithmetic identical on x86 and Arm
CFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    exe = shutil.which("nvcc")
    if exe is None:
        cand = Path("/usr/local/cuda/bin/nvcc")
        if cand.exists():
            return str(cand)
        raise RuntimeError("nvcc not found: the melvin GB300 library cannot be built")
    return exe


def lib_path() -> Path:
    return LIB_DIR / LIB_NAME


def _newest_header() -> float:
    hs = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: Path, obj: Path, extra: list[str]) -> tuple[Path, str]:
    cmd = [nvcc()] + ARCH + CFLAGS + extra + ["-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src.name}:\n{res.stdout}\n{res.stderr}")
    return obj, res.stderr


def build(verbose: bool = False, jobs: int | None = None, extra_flags: list[str] | None = None) -> Path:
    """Compile and link the library; returns its path."""
    extra = list(extra_flags or [])
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB_DIR.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    if not sources:
        raise RuntimeError(f"no CUDA sources under {CSRC}")
    hdr = _newest_header()
    todo = []
    objs = []
    for src in sources:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, hdr):
            todo.append((src, obj))
    # Compile the largest translation units first.
    todo.sort(key=lambda t: -t[0].stat().st_size)
    workers = jobs or max(1, min(len(todo), os.cpu_count() or 1))
    if todo:
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            futs = [ex.submit(_compile, s, o, extra) for s, o in todo]
            for f in cf.as_completed(futs):
                obj, log = f.result()
                if verbose and log.strip():
                    print(f"[{obj.name}]\n{log}", file=sys.stderr)
    out = lib_path()
    if (not out.exists()) or todo or out.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        tmp = out.with_suffix(".so.tmp")
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", str(tmp)] + [str(o) for o in objs]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, out)
    return out


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
