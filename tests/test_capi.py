"""CPU checks of the C ABI library: it loads, exports every symbol the header
declares, and its host-only entry points (parameter setup, initial-condition
generator, argument validation) behave like the reference's para.f90 and the
oracle.  No call here launches GPU work."""
from __future__ import annotations

import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

HEADER = Path(__file__).resolve().parents[1] / "include" / "lbm_gb300.h"


def declared_functions() -> list[str]:
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lbm_[a-z_0-9]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib, pkg):
    names = declared_functions()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(pkg.EXPORTS) == names


def test_library_build_targets_sm103a_only():
    """The build recipe compiles every translation unit for sm_103a alone."""
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "lbm_gb300_build", Path(__file__).resolve().parents[1] / "d3q19-single-phase_gb300" / "_build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert all(a in b.NVCC_FLAGS for a in b.ARCH)


def test_params_init_matches_para(lib, pkg):
    for mrt in (1, 2, 3):
        run = pkg.RunParams(nx=64, ny=128, nz=64, visc=0.0012, force_y=3.8e-7, mrt_type=mrt)
        c = run.to_c()
        r = run.rates()
        for k, v in r.items():
            assert getattr(c, k) == pytest.approx(v, rel=1e-15), (mrt, k)
        assert list(c.force) == [0.0, 3.8e-7, 0.0]
        assert c.fp16_scale == 32768.0


def test_params_init_rejects_bad_arguments(lib, pkg):
    p = pkg.LBMParams()
    assert lib.lbm_params_init(ctypes.byref(p), 0, 4, 4, 1, 0.01, 0.0, 0) == -1
    assert lib.lbm_params_init(ctypes.byref(p), 4, 4, 4, 7, 0.01, 0.0, 0) == -1
    assert lib.lbm_params_init(ctypes.byref(p), 4, 4, 4, 1, -1.0, 0.0, 0) == -1
    assert lib.lbm_params_init(ctypes.byref(p), 4, 4, 4, 1, 0.01, 0.0, 5) == -1
    assert b"MRT" in lib.lbm_last_error() or b"precision" in lib.lbm_last_error()
    assert lib.lbm_params_init(None, 4, 4, 4, 1, 0.01, 0.0, 0) == -1


def test_create_rejects_bad_params_before_touching_a_device(lib, pkg):
    p = pkg.LBMParams()
    assert lib.lbm_params_init(ctypes.byref(p), 4, 4, 4, 1, 0.01, 0.0, 0) == 0
    ctx = ctypes.c_void_p()
    p.nx = -3
    assert lib.lbm_create(ctypes.byref(p), ctypes.byref(ctx)) == -1
    assert not ctx.value
    p.nx = 4
    p.s9 = float("nan")
    assert lib.lbm_create(ctypes.byref(p), ctypes.byref(ctx)) == -1
    assert lib.lbm_create(None, ctypes.byref(ctx)) == -1
    assert lib.lbm_destroy(None) == 0
    assert lib.lbm_step(None, 1) == -1


def test_strerror_covers_codes(lib):
    for code in range(0, -9, -1):
        assert lib.lbm_strerror(code)
    assert lib.lbm_strerror(-99) == b"unknown error"


def test_channel_velocity_host_copy_matches_oracle(pkg, orc):
    for shape, seed in (((6, 5, 4), 1), ((16, 8, 4), 20240611)):
        a = pkg.channel_velocity(*shape, 0.05, 0.05, seed)
        b = orc.channel_velocity(*shape, 0.05, 0.05, seed)
        for x, y in zip(a, b):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("shape,a9", [((64, 32, 16), 0.0), ((63, 20, 12), 1.5)])
def test_loglaw_velocity_host_copy_matches_oracle(pkg, orc, shape, a9):
    """The library's table form of initvel (transcendentals per wall plane and
    per column) gives the bits of the oracle's literal loops."""
    ustar, visc = 0.0035, 0.0012
    a = pkg.loglaw_velocity(*shape, ustar, visc / ustar, a9)
    b = orc.loglaw_velocity(*shape, ustar, visc / ustar, a9)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_loglaw_velocity_rejects_bad_arguments(lib):
    buf = (ctypes.c_double * 64)()
    assert lib.lbm_loglaw_velocity(4, 4, 4, ctypes.c_double(0.0), ctypes.c_double(1.0), ctypes.c_double(0.0),
                                   buf, buf, buf) == -1
    assert lib.lbm_loglaw_velocity(4, 4, 4, ctypes.c_double(0.1), ctypes.c_double(float("nan")),
                                   ctypes.c_double(0.0), buf, buf, buf) == -1
    assert lib.lbm_init_loglaw(None, ctypes.c_double(0.1), ctypes.c_double(1.0), ctypes.c_double(0.0)) == -1


def test_les_wall_damping_rejects_bad_arguments(lib):
    assert lib.lbm_les_wall_damping(None, ctypes.c_double(26.0)) == -1
    assert lib.lbm_prerelax(None, None, None, None, ctypes.c_double(1e-5), 10, None, None) == -1


def test_oracle_sphere_placement_matches_library(pkg, orc):
    """The oracle restates the seeded placement (its plain all-pairs overlap
    scan against the library's cell list): the same centres bit for bit, so
    the CPU baseline runs the same geometry without the product library."""
    for args, seed in (((64, 64, 64, 16, 8.0), 12345), ((64, 128, 128, 256, 4.0), 7),
                       ((128, 256, 128, 256, 8.0), 99)):
        a = orc.place_spheres(*args, gap=2.0, wall_gap=1.0, seed=seed)
        b = pkg.place_spheres(*args, gap=2.0, wall_gap=1.0, seed=seed)
        assert np.array_equal(a, b)
    with pytest.raises(ValueError):
        orc.place_spheres(16, 16, 16, 50, 6.0)


def test_channel_configs(pkg):
    ch = pkg.CHANNEL_CONFIGS["channel-128x64x64"]
    assert (ch.wall, ch.stream, ch.span) == (64, 128, 64)
    assert ch.force == pytest.approx(0.0035**2 / 32)
    p = ch.params()
    assert (p.nx, p.ny, p.nz) == (64, 128, 64)
    big = pkg.CHANNEL_CONFIGS["spheres-1024x512x512"]
    assert big.nodes == 1024 * 512 * 512 and big.precision == "fp16"


def test_driver_creates_its_output_directory(tmp_path):
    """channel_gb300 creates its output directory and parents first, as the
    reference's para makes its output directories (makedir, para.f90:311-317);
    the run itself needs a GPU, so only the directory is checked here."""
    drv = Path(__file__).resolve().parents[1] / "d3q19-single-phase_gb300" / "channel_gb300"
    if not drv.exists():
        pytest.skip("driver not built")
    out = tmp_path / "runs" / "c0"
    subprocess.run([str(drv), f"out={out}", "nx=4", "ny=8", "nz=4", "steps=0"], capture_output=True, timeout=120)
    assert out.is_dir()
