"""GPU parity: the sm_103a kernels, called through the C ABI, against the FP64
oracle and the committed golden fixtures.

Tolerances
  FP64 storage + arithmetic: relative L-infinity <= 1e-10 in f, rho and u after
    100 steps (the parity bar of the FP64 path); the kernels reorder the same FP64
    arithmetic, so the observed gap is ~1e-14.
  FP32 and FP16 storage (FP32 arithmetic): checked against FP64 through the
    mean profile and bounded population errors, see test_precision_*.
"""
from __future__ import annotations

import os
import tempfile
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = Path(__file__).resolve().parent / "golden" / "channel_6x10x4.npz"


def rel_linf(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def stable_run(pkg, shape, force_y=3.8e-7, precision="fp64", visc=0.0012, mrt=1):
    nx, ny, nz = shape
    return pkg.RunParams(nx=nx, ny=ny, nz=nz, visc=visc, force_y=force_y, mrt_type=mrt,
                         precision=pkg.PRECISIONS[precision])


def random_state(orc, shape, seed, amp=1e-4):
    u = orc.channel_velocity(*shape, 0.05, 0.05, seed)
    f = orc.initpop(*u)
    rng = np.random.default_rng(seed)
    return np.asfortranarray(f + amp * rng.standard_normal(f.shape))


def test_upload_download_roundtrip(pkg, orc):
    shape = (6, 33, 5)
    f = random_state(orc, shape, 1)
    for prec, tol in (("fp64", 0.0), ("fp32", 6e-8), ("fp16", 5e-4)):
        with pkg.Lattice(stable_run(pkg, shape, precision=prec)) as lat:
            lat.upload_f(f)
            g = lat.download_f()
            err = np.abs(g - f)
            assert (err <= tol * np.abs(f) + 1e-12 * (prec == "fp16")).all(), prec


def test_device_initial_condition_is_bitwise_oracle_initpop(pkg, orc):
    shape = (8, 40, 6)
    with pkg.Lattice(stable_run(pkg, shape)) as lat:
        lat.init_channel(0.05, 0.05, 77)
        g = lat.download_f()
        u = orc.channel_velocity(*shape, 0.05, 0.05, 77)
        assert np.array_equal(g, orc.initpop(*u))
        # host-array initpop gives the same bits too
        lat.initpop(*u)
        assert np.array_equal(lat.download_f(), g)


@pytest.mark.parametrize("shape,a9", [((8, 40, 6), 0.0), ((9, 24, 10), 1.5), ((64, 32, 16), 0.7)])
def test_device_loglaw_initial_condition_is_bitwise_oracle(pkg, orc, shape, a9):
    """initvel's turbulent start (initial.f90:101-147) + initpop on the device
    equals the oracle's literal restatement bit for bit, the perturbation
    (A9 != 0) and an odd wall-normal size (untouched middle plane) included;
    lbm_prerelax takes the host copy of the same field."""
    ustar = 0.0035
    ystar = 0.0012 / ustar
    u = orc.loglaw_velocity(*shape, ustar, ystar, a9)
    want = orc.initpop(*u)
    with pkg.Lattice(stable_run(pkg, shape)) as lat:
        lat.init_loglaw(ustar, ystar, a9)
        assert np.array_equal(lat.download_f(), want)
    for prec in ("fp32", "fp16"):
        with pkg.Lattice(stable_run(pkg, shape, precision=prec)) as lat:
            lat.init_loglaw(ustar, ystar, a9)
            g = lat.download_f()
        # one rounding of each stored deviation: half an ulp of the storage type
        # (FP16 holds 2^15 (f - w), 11 significant bits; subnormals below 2^-14)
        rel_ulp = 2.0**-24 if prec == "fp32" else 2.0**-11
        floor = 0.0 if prec == "fp32" else 2.0**-25 / 2**15
        assert (np.abs(g - want) <= 1.001 * rel_ulp * np.abs(want) + floor).all()


@pytest.mark.parametrize("nsteps", [1, 2, 3, 8])
def test_steps_match_oracle_fp64(pkg, orc, nsteps):
    shape = (6, 12, 5)
    run = stable_run(pkg, shape, force_y=2e-5)
    f = random_state(orc, shape, 10 + nsteps)
    fo, rho, ux, uy, uz = orc.run(orc.params_from(run), f, nsteps, mode=0)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f)
        lat.step(nsteps)
        g = lat.download_f()
        m = lat.macrovar()
    assert rel_linf(g, fo) < 1e-13
    for a, b in zip(m, (rho, ux, uy, uz)):
        assert rel_linf(a, b) < 1e-12


@pytest.mark.parametrize("shape", [(1, 4, 3), (2, 5, 1), (3, 1, 2), (7, 9, 11)])
def test_odd_shapes_match_oracle(pkg, orc, shape):
    run = stable_run(pkg, shape, force_y=1e-5)
    f = random_state(orc, shape, 3)
    fo = orc.run(orc.params_from(run), f, 5, mode=0)[0]
    with pkg.Lattice(run) as lat:
        lat.upload_f(f)
        lat.step(5)
        assert rel_linf(lat.download_f(), fo) < 1e-13


def test_golden_fixture(pkg):
    g = np.load(GOLDEN)
    nx, ny, nz = (int(v) for v in g["shape"])
    run = pkg.RunParams(nx=nx, ny=ny, nz=nz, visc=float(g["visc"]), force_y=float(g["force"][1]), mrt_type=1)
    with pkg.Lattice(run) as lat:
        lat.upload_f(g["f0"])
        done = 0
        for n in g["steps"]:
            lat.step(int(n) - done)
            done = int(n)
            assert rel_linf(lat.download_f(), g[f"f{n}"]) < 1e-13
            m = np.stack(lat.macrovar())
            assert rel_linf(m, g[f"macro{n}"]) < 1e-12


def test_config0_fp64_parity_100_steps(pkg, orc):
    """Plain turbulent channel 128 x 64 x 64 (ch), seeded Poiseuille + 5 %
    noise, 100 steps: relative L-inf <= 1e-10 in f, rho and u."""
    ch = pkg.CHANNEL_CONFIGS["channel-128x64x64"]
    run = ch.params("fp64")
    shape = (run.nx, run.ny, run.nz)
    u = orc.channel_velocity(*shape, ch.uc, ch.amp, ch.seed)
    f0 = orc.initpop(*u)
    p = orc.params_from(run)
    fo = orc.run_omp(p, np.array(f0, order="F", copy=True), 100, orc.max_threads())
    rho, ux, uy, uz = orc.macrovar(p, fo)
    with pkg.Lattice(run) as lat:
        lat.init_channel(ch.uc, ch.amp, ch.seed)
        assert np.array_equal(lat.download_f(), f0)
        lat.step(100)
        g = lat.download_f()
        m = lat.macrovar()
        prof = lat.profiles()
    errs = [rel_linf(g, fo)] + [rel_linf(a, b) for a, b in zip(m, (rho, ux, uy, uz))]
    assert max(errs) <= 1e-10, errs
    np.testing.assert_allclose(prof, orc.profiles(rho, ux, uy, uz), rtol=1e-9, atol=1e-13)


def test_prerelax_matches_oracle(pkg, orc):
    shape = (8, 16, 6)
    run = stable_run(pkg, shape)
    u = orc.channel_velocity(*shape, 0.05, 0.05, 5)
    f = orc.initpop(*u)
    f[0] += 1e-3 * np.random.default_rng(2).standard_normal(f.shape[1:])
    fo, it, err, rc = orc.prerelax(orc.params_from(run), f, *u, eps=1e-6, maxit=5000)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f)
        it2, err2 = lat.prerelax(*u, eps=1e-6, maxit=5000)
        assert it2 == it
        assert err2 == pytest.approx(err, rel=1e-6, abs=1e-15)
        assert rel_linf(lat.download_f(), fo) < 1e-12


def test_prerelax_with_velocity_from_the_populations(pkg, orc):
    """Pre-relaxation with the frozen velocity read back from the populations
    (no host arrays) equals the one given initvel's host arrays: the log-law
    start with a density disturbance in the rest population (which carries no
    momentum), same iteration count, populations to rounding."""
    shape = (12, 16, 8)
    run = stable_run(pkg, shape)
    ustar = 0.0035
    u = orc.loglaw_velocity(*shape, ustar, 0.0012 / ustar, 1.5)
    f = orc.initpop(*u)
    f[0] += 1e-3 * np.random.default_rng(4).standard_normal(f.shape[1:])
    out = []
    for host in (True, False):
        with pkg.Lattice(run) as lat:
            lat.upload_f(f)
            it, err = lat.prerelax(*(u if host else (None, None, None)), eps=1e-8, maxit=5000)
            out.append((it, err, lat.download_f()))
    assert out[0][0] == out[1][0] and out[0][0] > 1
    assert rel_linf(out[1][2], out[0][2]) < 1e-12


def test_prerelax_limit_reports_not_converged(pkg, orc):
    shape = (4, 8, 4)
    run = stable_run(pkg, shape)
    u = orc.channel_velocity(*shape, 0.05, 0.05, 5)
    f = orc.initpop(*u)
    f[0] += 1e-2
    with pkg.Lattice(run) as lat:
        lat.upload_f(f)
        with pytest.raises(pkg.LBMError) as e:
            lat.prerelax(*u, eps=1e-14, maxit=3)
        assert e.value.code == -5


def test_poiseuille_startup_on_gpu(pkg, orc):
    nx = 20
    run = pkg.para(nx, 4, 4, laminar=True)
    z = np.zeros((nx, 4, 4), order="F")
    with pkg.Lattice(run) as lat:
        lat.initpop(z, z, z)
        lat.step(120)
        rho, ux, uy, uz = lat.macrovar()
    ana = orc.poiseuille_transient(nx, run.ustar, run.visc, 120)
    assert np.abs(uy[: nx // 2, 1, 1] / run.ustar - ana).max() < 5e-3


def test_diag_and_mass_conservation(pkg, orc):
    ch = pkg.CHANNEL_CONFIGS["channel-128x64x64"]
    run = ch.params("fp64")
    with pkg.Lattice(run) as lat:
        lat.init_channel(ch.uc, ch.amp, ch.seed)
        st0 = lat.diag()
        lat.step(200)
        st = lat.diag()
        rho, ux, uy, uz = lat.macrovar()
    assert st.nfluid == ch.nodes and st.nonfinite == 0
    assert abs(st.rho_sum - st0.rho_sum) < 1e-9
    assert st.rho_max == pytest.approx(rho.max(), rel=1e-12)
    assert st.rho_min == pytest.approx(rho.min(), rel=1e-12)
    v = np.sqrt(ux**2 + uy**2 + uz**2)
    assert st.vmax == pytest.approx(v.max(), rel=1e-12)
    ix, iy, iz = np.unravel_index(np.argmax(v.ravel(order="F")), v.shape, order="F")
    assert tuple(st.vmax_at) == (ix + 1, iy + 1, iz + 1)
    assert st.mom_sum[1] == pytest.approx(uy.sum(), rel=1e-10)


def read_fortran_records(path):
    """Parse a gfortran-style unformatted sequential file into records."""
    data = Path(path).read_bytes()
    recs, pos = [], 0
    while pos < len(data):
        chunks = []
        while True:
            n = int(np.frombuffer(data, np.int32, 1, pos)[0])
            pos += 4
            chunks.append(data[pos:pos + abs(n)])
            pos += abs(n)
            pos += 4
            if n >= 0:
                break
        recs.append(b"".join(chunks))
    return recs


def test_checkpoint_files_in_reference_format(pkg, orc):
    shape = (6, 12, 5)
    run = stable_run(pkg, shape)
    f = random_state(orc, shape, 9)
    with tempfile.TemporaryDirectory() as d, pkg.Lattice(run) as lat:
        lat.upload_f(f)
        lat.step(3)                                  # odd step count: swapped AA state
        want = lat.download_f()
        p0 = os.path.join(d, "finit.000")
        p1 = os.path.join(d, "endrunflow2D16x8.0000003.000")
        lat.save_flow(p0, 0, [7])
        lat.save_flow(p1, 1, [3, 1, 0])
        r0 = read_fortran_records(p0)
        assert len(r0) == 2 and np.frombuffer(r0[0], np.int32).tolist() == [7]
        assert np.array_equal(np.frombuffer(r0[1], np.float64), want.ravel(order="F"))
        r1 = read_fortran_records(p1)
        assert np.frombuffer(r1[0], np.int32).tolist() == [3, 1, 0]
        lat.step(2)
        assert lat.load_flow(p1, 1) == [3, 1, 0]
        assert np.array_equal(lat.download_f(), want)
        # continuing from the file equals continuing without it
        lat.step(4)
        a = lat.download_f()
        lat.upload_f(want)
        lat.step(4)
        assert np.array_equal(lat.download_f(), a)
        # corrupt / wrong-size files are rejected with LBM_ERR_IO
        bad = os.path.join(d, "bad")
        Path(bad).write_bytes(Path(p0).read_bytes()[:-100])
        with pytest.raises(pkg.LBMError) as e:
            lat.load_flow(bad, 0)
        assert e.value.code == -6
        with pytest.raises(pkg.LBMError):
            lat.load_flow(os.path.join(d, "missing"), 0)
        with pytest.raises(pkg.LBMError):
            lat.load_flow(p1, 0)                     # header holds 3 integers, not 1


def test_precision_variants_against_fp64(pkg):
    """FP32 and FP16-storage runs of the ch channel against FP64 after 300
    steps: mean streamwise profile within 1 % and bounded population error."""
    ch = pkg.CHANNEL_CONFIGS["channel-128x64x64"]
    res = {}
    for prec in ("fp64", "fp32", "fp16"):
        with pkg.Lattice(ch.params(prec)) as lat:
            lat.init_channel(ch.uc, ch.amp, ch.seed)
            lat.step(300)
            res[prec] = (lat.profiles(), lat.download_f(), lat.diag())
    ref = pkg.statistics(res["fp64"][0], ch.ustar)
    for prec, tol_f in (("fp32", 1e-5), ("fp16", 2e-2)):
        st = pkg.statistics(res[prec][0], ch.ustar)
        err_mean = np.abs(st["mean"][:, 1] - ref["mean"][:, 1]).max() / np.abs(ref["mean"][:, 1]).max()
        assert err_mean < 1e-2, (prec, err_mean)
        assert rel_linf(res[prec][1], res["fp64"][1]) < tol_f, prec
        assert res[prec][2].nonfinite == 0


def test_avedensity_removes_mean(pkg, orc):
    shape = (6, 12, 5)
    run = stable_run(pkg, shape)
    f = random_state(orc, shape, 4)
    f[0] += 3e-4
    with pkg.Lattice(run) as lat:
        lat.upload_f(f)
        lat.step(1)
        m = lat.avedensity()
        assert m == pytest.approx(3e-4, rel=0.2)
        assert abs(lat.diag().rho_sum) < 1e-12


@pytest.mark.parametrize("prec", ["fp32", "fp16"])
@pytest.mark.parametrize("shape", [(5, 16, 3), (8, 64, 7), (3, 24, 1), (6, 32, 9), (4, 512, 3), (4, 1024, 3),
                                   (3, 1536, 2), (2, 3072, 2), (5, 16, 6), (4, 512, 4), (3, 256, 2)])
def test_row_pipelined_kernels_match_simple_kernels(pkg, orc, prec, shape):
    """The bulk-copy row kernels (FP32/FP16 storage, rows of 16-byte multiples)
    against the one-node-per-thread kernels: same arithmetic per node, so the
    populations agree to rounding of the storage type.  The streamwise rows
    cover the launch shapes: two CTAs of 256 threads with one row per item
    (short rows with an odd spanwise count, idle threads in each item; FP16
    rows of 1024, two pairs per thread) and with two rows per item (rows of
    up to 512 with an even spanwise count, including the pair of rows split
    by the periodic wrap), one CTA of 512 threads (FP16 rows of 1536, FP32
    of 1024), and rows too long for two stages, which run the
    one-node-per-thread kernels under either flag (FP16 3072, FP32 1536)."""
    f = random_state(orc, shape, 21)
    out = {}
    for flags in (0, pkg.FLAG_SIMPLE_STEP):
        run = stable_run(pkg, shape, force_y=2e-5, precision=prec)
        run.flags = flags
        with pkg.Lattice(run) as lat:
            lat.upload_f(f)
            res = []
            for n in (1, 1, 5):
                lat.step(n)
                res.append(lat.download_f())
            out[flags] = res
    ulp = 2.0**-23 if prec == "fp32" else 2.0**-10
    for a, b in zip(out[0], out[pkg.FLAG_SIMPLE_STEP]):
        assert np.abs(a - b).max() <= 4 * ulp * np.abs(b).max()
    # and both follow the FP64 oracle within the storage precision
    fo = orc.run(orc.params_from(stable_run(pkg, shape, force_y=2e-5)), f, 7, mode=0)[0]
    assert rel_linf(out[0][-1], fo) < (1e-5 if prec == "fp32" else 5e-3)


@pytest.mark.parametrize("prec", ["fp32", "fp16"])
def test_row_kernels_production_rows_match_oracle(pkg, orc, prec):
    """Rows of 1024 streamwise nodes, as in the large channel (FP16: two CTAs
    of 256 threads per SM with two stages each; FP32: one CTA of 512 threads),
    on a 1.6 M-node channel from the seeded Poiseuille start: 10 steps against
    the FP64 oracle (its OpenMP push), within the storage precision."""
    shape = (32, 1024, 48)                      # wall-normal, streamwise, spanwise
    run = stable_run(pkg, shape, force_y=2e-6, precision=prec)
    u = orc.channel_velocity(*shape, 0.05, 0.05, 31)
    f0 = orc.initpop(*u)
    p64 = orc.params_from(stable_run(pkg, shape, force_y=2e-6))
    fo = orc.run_omp(p64, f0.copy(order="F"), 10, orc.max_threads())    # fused two-lattice push, OpenMP
    _, _, uy_o, _ = orc.macrovar(p64, fo)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f0)
        lat.step(10)
        g = lat.download_f()
        rho, ux, uy, uz = lat.macrovar()
    tol = 1e-5 if prec == "fp32" else 5e-3
    assert rel_linf(g, fo) < tol
    assert rel_linf(uy, uy_o) < tol
    assert abs(float(g.sum() - fo.sum())) < tol * np.abs(fo).sum()


def test_row_kernels_full_size_config4_properties(pkg):
    """1024 x 512 x 512 FP16 store (the large channel): no NaN, mass drift and
    mean profile against the one-node-per-thread kernels after 20 steps."""
    big = pkg.CHANNEL_CONFIGS["spheres-1024x512x512"]
    res = {}
    for flags in (0, pkg.FLAG_SIMPLE_STEP):
        run = big.params("fp16")
        run.flags = flags
        with pkg.Lattice(run) as lat:
            lat.init_channel(big.uc, big.amp, big.seed)
            d0 = lat.diag()
            lat.step(20)
            d1 = lat.diag()
            res[flags] = (lat.profiles(), d1, d1.rho_sum - d0.rho_sum)
    a, b = res[0], res[pkg.FLAG_SIMPLE_STEP]
    assert a[1].nonfinite == 0 and b[1].nonfinite == 0
    ma = pkg.statistics(a[0], big.ustar)["mean"][:, 1]
    mb = pkg.statistics(b[0], big.ustar)["mean"][:, 1]
    assert np.abs(ma - mb).max() < 1e-4 * np.abs(mb).max()
    assert abs(a[2]) < 1e-5 * big.nodes and abs(b[2]) < 1e-5 * big.nodes
