"""Build the in-tree CUDA library ``liblbm_gb300.so`` for sm_103a.

The library holds every kernel of the time step and the ``extern "C"``
boundary declared in ``include/lbm_gb300.h``.  Translation units are compiled
in parallel with nvcc and linked into the package directory; nothing is
installed into site-packages.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
REPO = PKG_DIR.parent
CSRC = PKG_DIR / "csrc"
OBJ_DIR = PKG_DIR / "_build"
LIB_PATH = PKG_DIR / "liblbm_gb300.so"
# bounds-checked variant (-DLBM_BOUNDS_CHECK): every checked index that falls
# outside its array is reported by the call that ran the kernel; for tests on
# small lattices, not for timing
DEBUG_OBJ_DIR = PKG_DIR / "_build_debug"
DEBUG_LIB_PATH = PKG_DIR / "liblbm_gb300_debug.so"
HOST_DIR = PKG_DIR / "host"
DRIVER_PATH = PKG_DIR / "channel_gb300"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    "-O3", "-std=c++17", "-lineinfo", *ARCH,
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "--expt-relaxed-constexpr",
]
SOURCES = ["lbm_step.cu", "lbm_step_tma.cu", "lbm_fields.cu", "lbm_particles.cu", "lbm_capi.cu", "lbm_noalloc.cu",
           "lbm_mlp.cu"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbm_gb300.so")
    return exe


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + [REPO / "include" / "lbm_gb300.h"]


def _stale(target: Path, inputs: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(p.stat().st_mtime > t for p in inputs)


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"command failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def build_library(force: bool = False, verbose: bool = False, debug: bool = False) -> Path:
    """Compile and link liblbm_gb300.so (debug: the bounds-checked
    liblbm_gb300_debug.so) if any source changed; return its path."""
    obj_dir = DEBUG_OBJ_DIR if debug else OBJ_DIR
    lib_path = DEBUG_LIB_PATH if debug else LIB_PATH
    defines = ["-DLBM_BOUNDS_CHECK"] if debug else []
    obj_dir.mkdir(exist_ok=True)
    exe = nvcc()
    deps = _deps()
    jobs = []
    objs = []
    for src in SOURCES:
        s = CSRC / src
        o = obj_dir / (src + ".o")
        objs.append(o)
        if force or _stale(o, [s, *deps]):
            extra = ["-Xptxas", "-v"] if verbose and src.endswith(".cu") else []
            jobs.append([exe, *NVCC_FLAGS, *defines, *extra, "-I", str(REPO / "include"), "-c", str(s),
                         "-o", str(o)])
    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 1)) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or _stale(lib_path, objs):
        tmp = lib_path.with_suffix(".so.tmp")
        _run([exe, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"])
        os.replace(tmp, lib_path)
    return lib_path


def build_driver(force: bool = False) -> Path:
    """Compile the C++ channel driver (mirror of the reference's main.f90)."""
    lib = build_library()
    src = HOST_DIR / "channel_main.cpp"
    if force or _stale(DRIVER_PATH, [src, lib, REPO / "include" / "lbm_gb300.h"]):
        cxx = shutil.which("g++") or "g++"
        _run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(REPO / "include"), str(src),
              "-o", str(DRIVER_PATH), "-L", str(PKG_DIR), "-llbm_gb300", f"-Wl,-rpath,{PKG_DIR}"])
    return DRIVER_PATH
