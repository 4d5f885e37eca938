"""The bounds-checked build on small lattices.

liblbm_gb300_debug.so is the same library compiled with -DLBM_BOUNDS_CHECK:
the bulk-copy row kernels check every source/destination row and each
pair's stream positions, the bounce-back kernel its staged box indices and
the global node of every gather and scatter, the ownership and refill
kernels their node indices.  A failing check records its site and skips the
access; the call that ran the kernel then fails with LBM_ERR_STATE, so a
clean run here means no checked index left its array.  The checked build
must also give the normal build's results: bit for bit in FP64 storage (the
particle arithmetic uses explicitly rounded FP64 operations), to rounding of
the storage type otherwise.
"""
from __future__ import annotations

import importlib.util
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

REPO = Path(__file__).resolve().parents[1]


@pytest.fixture(scope="module")
def debug_lib(pkg):
    spec = importlib.util.spec_from_file_location("lbm_gb300_build", REPO / "d3q19-single-phase_gb300" / "_build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return pkg.load_library(b.build_library(debug=True))


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def run_both(pkg, debug_lib, run, f0, steps, pos=None, vel=None, radius=4.0):
    out = []
    for lib in (None, debug_lib):
        with pkg.Lattice(run, lib=lib) as lat:
            lat.upload_f(f0)
            if pos is not None:
                lat.set_particles(pos, radius=radius, rho_ratio=2.0, vel=vel)
            res = []
            for n in steps:
                lat.step(n)                      # raises on a failed bounds check
                res.append(lat.download_f())
            part = lat.particles() if pos is not None else None
        out.append((res, part))
    return out


@pytest.mark.parametrize("prec", ["fp32", "fp16"])
@pytest.mark.parametrize("shape", [(5, 16, 3), (3, 24, 1), (6, 32, 9), (4, 1024, 3), (3, 1536, 2), (4, 512, 4),
                                   (5, 16, 6)])
def test_row_kernels_checked(pkg, orc, debug_lib, prec, shape):
    nx, ny, nz = shape
    run = pkg.RunParams(nx=nx, ny=ny, nz=nz, visc=0.0012, force_y=2e-5, mrt_type=1, precision=pkg.PRECISIONS[prec])
    f0 = orc.initpop(*orc.channel_velocity(*shape, 0.05, 0.05, 5))
    (a, _), (b, _) = run_both(pkg, debug_lib, run, f0, (1, 1, 4))
    ulp = 2.0**-23 if prec == "fp32" else 2.0**-10
    for x, y in zip(a, b):
        assert np.abs(x - y).max() <= 4 * ulp * np.abs(x).max()


@pytest.mark.parametrize("prec,radius", [("fp64", 4.0), ("fp16", 4.0), ("fp32", 12.0)])
def test_sphere_kernels_checked(pkg, orc, debug_lib, prec, radius):
    """Three moving spheres (one crossing the periodic streamwise edge) and,
    at radius 12, the 64-bit staged rows; 26 steps cover both AA parities,
    refills and the release/claim shell."""
    shape = (24, 32, 22) if radius == 4.0 else (32, 40, 40)
    if radius == 4.0:
        pos = np.array([[8.3, 30.2, 7.7], [15.6, 21.9, 13.1], [12.0, 4.4, 16.8]])
        vel = np.array([[0.0, 0.01, 0.0], [0.002, -0.003, 0.001], [0.0, 0.0, 0.004]])
    else:
        pos = np.array([[16.2, 39.0, 20.4]])
        vel = np.array([[0.001, 0.004, -0.002]])
    nx, ny, nz = shape
    run = pkg.RunParams(nx=nx, ny=ny, nz=nz, visc=0.02, force_y=2e-6, mrt_type=1, precision=pkg.PRECISIONS[prec])
    f0 = orc.initpop(*orc.channel_velocity(*shape, 0.04, 0.05, 3))
    (a, pa), (b, pb) = run_both(pkg, debug_lib, run, f0, (1, 25), pos, vel, radius)
    if prec == "fp64":
        for x, y in zip(a, b):
            assert rel(y, x) < 1e-14
        for k in ("pos", "vel", "force", "torque"):
            assert rel(pb[k], pa[k]) < 1e-12, k
    else:
        for x, y in zip(a, b):
            assert rel(y, x) < 1e-3
        assert rel(pb["force"], pa["force"]) < 1e-2
