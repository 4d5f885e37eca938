"""CPU checks of the FP64 oracle: lattice algebra, collision known answers,
the reference's swap/exchange semantics against an independent push, the
analytic Poiseuille start-up (the reference's only known answer,
saveload.f90:920-936), pre-relaxation and the seeded initial condition."""
from __future__ import annotations

import numpy as np
import pytest

RNG = np.random.default_rng(12345)


def lbgk_rates(visc=0.05):
    s9 = 1.0 / (3 * visc + 0.5)
    return dict(s1=s9, s2=s9, s4=s9, s9=s9, s10=s9, s13=s9, s16=s9, omegepsl=3.0, omegepslj=-5.5, omegxx=-0.5)


def stable_rates(visc=0.0012):
    s9 = 1.0 / (3 * visc + 0.5)
    return dict(s1=1.5, s2=1.4, s4=1.2, s9=s9, s10=1.4, s13=s9, s16=1.98,
                omegepsl=0.0, omegepslj=-475.0 / 63.0, omegxx=0.0)


def random_f(orc, shape, amp=0.02, seed=0):
    rng = np.random.default_rng(seed)
    u = [0.05 * rng.uniform(-1, 1, shape) for _ in range(3)]
    f = orc.initpop(*u)
    return f + amp * 0.01 * rng.standard_normal(f.shape)


def test_moment_matrix_is_dhumieres_basis(orc):
    M, d = orc.moment_matrix()
    # orthogonal rows with the squared norms the back-transform divides by
    # (val1..val9 = 19, 2394, 252, 10, 40, 36, 72, 12, 24; 1/coef4i = 4; coef3 = 8)
    G = M @ M.T
    assert np.array_equal(G, np.diag(np.diag(G)))
    expect = [19, 2394, 252, 10, 40, 10, 40, 10, 40, 36, 72, 12, 24, 4, 4, 4, 8, 8, 8]
    assert np.array_equal(d, np.array(expect, dtype=float))
    assert np.array_equal(M[3], orc.CX) and np.array_equal(M[5], orc.CY) and np.array_equal(M[7], orc.CZ)


def closed_form_force_moments(F, u):
    """M Fbar in closed form, the expression the GPU kernel uses."""
    Fx, Fy, Fz = F
    ux, uy, uz = u
    A = ux * Fx + uy * Fy + uz * Fz
    P = 2 * ux * Fx - uy * Fy - uz * Fz
    W = uy * Fy - uz * Fz
    return np.array([0, 38 * A, -11 * A, Fx, -2 / 3 * Fx, Fy, -2 / 3 * Fy, Fz, -2 / 3 * Fz,
                     2 * P, -P, 2 * W, -W, Fx * uy + Fy * ux, Fy * uz + Fz * uy, Fx * uz + Fz * ux, 0, 0, 0])


def test_force_moments_closed_form(orc):
    for _ in range(20):
        F = RNG.uniform(-1e-3, 1e-3, 3)
        u = RNG.uniform(-0.1, 0.1, 3)
        p = orc.params(stable_rates(), F)
        mf = orc.force_moments(p, *u)
        np.testing.assert_allclose(mf, closed_form_force_moments(F, u), rtol=0, atol=1e-17)


def test_collision_with_unit_rates_gives_equilibrium_plus_half_force(orc):
    # 1-node KAT: with every rate 1 and the LBGK equilibrium coefficients the
    # MRT collision returns the second-order equilibrium plus Fbar/2.
    r = dict(s1=1.0, s2=1.0, s4=1.0, s9=1.0, s10=1.0, s13=1.0, s16=1.0, omegepsl=3.0, omegepslj=-5.5,
             omegxx=-0.5)
    F = np.array([1e-4, -2e-4, 3e-5])
    p = orc.params(r, F)
    f = random_f(orc, (1, 1, 1))[:, 0, 0, 0]
    rho = f.sum()
    u = np.array([orc.CX @ f, orc.CY @ f, orc.CZ @ f]) + F / 2
    out = orc.collide_node(p, f, rho, *u)
    cu = orc.CX * u[0] + orc.CY * u[1] + orc.CZ * u[2]
    feq = orc.W * (rho + 3 * cu + 4.5 * cu**2 - 1.5 * (u @ u))
    uF = u @ F
    cF = orc.CX * F[0] + orc.CY * F[1] + orc.CZ * F[2]
    Fbar = orc.W * (3 * cF + 9 * cF * cu - 3 * uF)
    np.testing.assert_allclose(out, feq + 0.5 * Fbar, rtol=0, atol=1e-16)


def test_collision_conserves_mass_and_adds_force(orc):
    F = np.array([0.0, 3.8e-7, 0.0])
    p = orc.params(stable_rates(), F)
    for k in range(10):
        f = random_f(orc, (1, 1, 1), seed=k)[:, 0, 0, 0]
        rho = f.sum()
        jf = np.array([orc.CX @ f, orc.CY @ f, orc.CZ @ f])
        out = orc.collide_node(p, f, rho, *(jf + F / 2))
        assert abs(out.sum() - rho) < 1e-16
        jo = np.array([orc.CX @ out, orc.CY @ out, orc.CZ @ out])
        np.testing.assert_allclose(jo, jf + F, rtol=0, atol=1e-17)


def gpu_collide_restated(f, F, r, frozen_u=None):
    """Float64 transcription of the moment-space update in
    csrc/lbm_collide.cuh (scale 1): checks the kernel's algebra on the CPU."""
    f = np.array(f, dtype=np.float64)
    s = {i: f[i] + f[j] for i, j in ((1, 2), (3, 4), (5, 6), (7, 10), (8, 9), (11, 14), (12, 13), (15, 18), (16, 17))}
    d = {i: f[i] - f[j] for i, j in ((1, 2), (3, 4), (5, 6), (7, 10), (8, 9), (11, 14), (12, 13), (15, 18), (16, 17))}
    syz5 = s[3] + s[5]
    sa = s[1] + syz5
    sxy, sxz, syz = s[7] + s[8], s[11] + s[12], s[15] + s[16]
    sd = sxy + sxz + syz
    rho = f[0] + (sa + sd)
    Dx = (d[7] - d[8]) + (d[11] - d[12])
    Dy = (d[7] + d[8]) + (d[15] - d[16])
    Dz = (d[11] + d[12]) + (d[15] + d[16])
    jf = np.array([d[1] + Dx, d[3] + Dy, d[5] + Dz])
    Fx, Fy, Fz = F
    j = jf + 0.5 * np.asarray(F) if frozen_u is None else np.asarray(frozen_u)
    jx, jy, jz = j
    ux, uy, uz = j
    ju = jx * ux + jy * uy + jz * uz
    A = jx * Fx + jy * Fy + jz * Fz
    P = 2 * jx * Fx - jy * Fy - jz * Fz
    Wf = jy * Fy - jz * Fz
    Qxy, Qyz, Qxz = jx * Fy + jy * Fx, jy * Fz + jz * Fy, jx * Fz + jz * Fx
    e = -30 * f[0] - 11 * sa + 8 * sd
    eps = 12 * f[0] - 4 * sa + sd
    q = np.array([-4 * d[1] + Dx, -4 * d[3] + Dy, -4 * d[5] + Dz])
    p3 = (2 * s[1] - syz5) + (sxy + sxz - 2 * syz)
    pi3 = (2 * syz5 - 4 * s[1]) + (sxy + sxz - 2 * syz)
    pw = (s[3] - s[5]) + (sxy - sxz)
    piw = -2 * (s[3] - s[5]) + (sxy - sxz)
    pxy, pyz, pxz = s[7] - s[8], s[15] - s[16], s[11] - s[12]
    mx = (d[7] - d[8]) - (d[11] - d[12])
    my = (d[15] - d[16]) - (d[7] + d[8])
    mz = (d[11] + d[12]) - (d[15] + d[16])
    eqp = 3 * jx * ux - ju
    eqw = jy * uy - jz * uz
    a_e = A * 38 / 2394 - r["s1"] / 2394 * (e + 19 * A + 11 * rho - 19 * ju)
    a_eps = A * -11 / 252 - r["s2"] / 252 * (eps - 5.5 * A - r["omegepsl"] * rho - r["omegepslj"] * ju)
    a_q = -(2 / 3) * np.asarray(F) / 40 - r["s4"] / 40 * (q + (2 / 3) * j - np.asarray(F) / 3)
    a_p = P * 2 / 36 - r["s9"] / 36 * (p3 + P - eqp)
    a_pi = P * -1 / 72 - r["s10"] / 72 * (pi3 - 0.5 * P - r["omegxx"] * eqp)
    a_w = Wf * 2 / 12 - r["s9"] / 12 * (pw + Wf - eqw)
    a_wi = Wf * -1 / 24 - r["s10"] / 24 * (piw - 0.5 * Wf - r["omegxx"] * eqw)
    a_xy = Qxy / 4 - r["s13"] / 4 * (pxy + 0.5 * Qxy - jx * uy)
    a_yz = Qyz / 4 - r["s13"] / 4 * (pyz + 0.5 * Qyz - jy * uz)
    a_xz = Qxz / 4 - r["s13"] / 4 * (pxz + 0.5 * Qxz - jx * uz)
    a_m = -r["s16"] / 8 * np.array([mx, my, mz])
    aj = np.asarray(F) / 10 if frozen_u is None else (j + 0.5 * np.asarray(F) - jf) / 10
    # back-transform as an explicit M^T a (a_k per moment)
    a = np.zeros(19)
    a[1], a[2] = a_e, a_eps
    a[3], a[5], a[7] = aj
    a[4], a[6], a[8] = a_q
    a[9], a[10], a[11], a[12] = a_p, a_pi, a_w, a_wi
    a[13], a[14], a[15] = a_xy, a_yz, a_xz
    a[16:19] = a_m
    return a, rho, j


def test_gpu_kernel_algebra_matches_oracle(orc):
    M, _ = orc.moment_matrix()
    for rates in (stable_rates(), lbgk_rates()):
        F = np.array([2e-6, 3.8e-7, -1e-6])
        p = orc.params(rates, F)
        for k in range(10):
            f = random_f(orc, (1, 1, 1), seed=100 + k)[:, 0, 0, 0]
            a, rho, j = gpu_collide_restated(f, F, rates)
            mine = f + M.T @ a
            ref = orc.collide_node(p, f, rho, *j)
            np.testing.assert_allclose(mine, ref, rtol=0, atol=2e-17)
            # frozen-velocity variant (pre-relaxation)
            uf = RNG.uniform(-0.05, 0.05, 3)
            a, rho, j = gpu_collide_restated(f, F, rates, frozen_u=uf)
            np.testing.assert_allclose(f + M.T @ a, orc.collide_node(p, f, rho, *uf), rtol=0, atol=2e-17)


@pytest.mark.parametrize("shape", [(4, 4, 4), (5, 6, 7), (1, 3, 2), (2, 1, 1), (3, 2, 1), (6, 5, 3)])
def test_swap_sweep_equals_push(orc, shape):
    """The reference's in-place swap sweep with its exchange rules, run on one
    rank that is its own periodic neighbour, equals an independent two-lattice
    push bit for bit (NaN-filled exchange buffers catch any unwritten slot)."""
    p = orc.params(stable_rates(), (0.0, 3.8e-7, 1e-7))
    f = random_f(orc, shape, seed=sum(shape))
    rho, ux, uy, uz = orc.macrovar(p, f)
    a = orc.step_swap(p, f, rho, ux, uy, uz)
    b = orc.step_push(p, f, rho, ux, uy, uz)
    assert np.isfinite(a).all()
    assert np.array_equal(a, b)


def test_run_modes_agree_over_many_steps(orc):
    p = orc.params(stable_rates(), (0.0, 3.8e-7, 0.0))
    f = random_f(orc, (6, 8, 4), seed=7)
    ra = orc.run(p, f, 9, mode=0)
    rb = orc.run(p, f, 9, mode=1)
    for x, y in zip(ra, rb):
        assert np.array_equal(x, y)


def test_streaming_is_a_permutation_with_walls(orc):
    """With every rate zero and no force the collision is the identity (up to
    the rounding of M^T D^-1 M), so a step is pure streaming: periodic in y/z,
    half-way bounce-back in x."""
    r = {k: 0.0 for k in ("s1", "s2", "s4", "s9", "s10", "s13", "s16", "omegepsl", "omegepslj", "omegxx")}
    p = orc.params(r)
    nx, ny, nz = 4, 5, 3
    f = RNG.standard_normal((19, nx, ny, nz))
    f = np.asfortranarray(f)
    rho, ux, uy, uz = orc.macrovar(p, f)
    g = orc.step_swap(p, f, rho, ux, uy, uz)
    for i in range(19):
        for ix in range(nx):
            xs = ix - orc.CX[i]
            for iy in range(ny):
                for iz in range(nz):
                    if 0 <= xs < nx:
                        src = f[i, xs, (iy - orc.CY[i]) % ny, (iz - orc.CZ[i]) % nz]
                    else:
                        src = f[orc.OPP[i], ix, iy, iz]
                    assert abs(g[i, ix, iy, iz] - src) <= 2e-15 * max(1.0, abs(src))


def test_poiseuille_startup_matches_analytic_series(orc):
    """Laminar channel of para.f90:74-88 from rest: the streamwise profile
    follows the 26-term series of outputuy (saveload.f90:921-933)."""
    nx = 20
    ustar = 0.05
    visc = 2.0 * ustar * nx / 20.0
    force = 8.0 * visc * ustar / nx**2
    p = orc.params(lbgk_rates(visc), (0.0, force, 0.0))
    z = np.zeros((nx, 2, 2), order="F")
    f = orc.initpop(z, z, z)
    errs = []
    for steps in (40, 120, 400):
        fo, rho, ux, uy, uz = orc.run(p, f, steps, mode=1)
        lbm = uy[: nx // 2, 0, 0] / ustar
        ana = orc.poiseuille_transient(nx, ustar, visc, steps)
        errs.append(np.abs(lbm - ana).max())
    # discretisation error of the lattice scheme, well below 1 % of u_c
    assert max(errs) < 5e-3, errs
    # steady state: the parabola of saveload.f90:926 up to the uniform slip
    # that LBGK with half-way bounce-back has at tau != 1/2 + sqrt(3/16)
    fo, rho, ux, uy, uz = orc.run(p, f, 6000, mode=1)
    xx0 = np.abs(np.arange(1, nx + 1) - 0.5 - nx / 2)
    uuss = 4 * ustar / nx**2 * ((nx / 2) ** 2 - xx0**2)
    slip = uy[:, 0, 0] - uuss
    assert np.abs(slip).max() < 0.02 * ustar
    assert np.ptp(slip) < 1e-3 * np.abs(slip).max()


def test_prerelax_exits_after_one_collision_from_equilibrium(orc):
    """initpop gives sum f = 0 = rho, so main.f90:70-90 exits on its first
    residual check (istep stays 0) after one collision."""
    p = orc.params(stable_rates(), (0.0, 3.8e-7, 0.0))
    u = orc.channel_velocity(8, 6, 4, 0.05, 0.05, 3)
    f = orc.initpop(*u)
    g, iters, err, rc = orc.prerelax(p, f, *u)
    assert rc == 0 and iters == 0 and err < 1e-15
    # and that one iteration is a step with the velocity frozen at u and
    # rho = sum f accumulated in population order (rhoupdat)
    rho = f[0].copy()
    for i in range(1, 19):
        rho += f[i]
    h = orc.step_swap(p, f, rho, *u)
    assert np.array_equal(g, h)


def test_prerelax_iterates_until_converged(orc):
    p = orc.params(stable_rates(), (0.0, 3.8e-7, 0.0))
    u = orc.channel_velocity(8, 6, 4, 0.05, 0.05, 3)
    f = orc.initpop(*u)
    f[0] += 1e-3 * np.random.default_rng(1).standard_normal(f.shape[1:])   # density perturbation
    g, iters, err, rc = orc.prerelax(p, f, *u, eps=1e-6, maxit=5000)
    assert rc == 0 and iters > 0 and err <= 1e-6


def numpy_uniform_pm1(seed, key):
    M = (1 << 64) - 1
    z = (seed * 0xD1B54A32D192ED03 + key) & M
    z = (z + 0x9E3779B97F4A7C15) & M
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & M
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & M
    z ^= z >> 31
    return (z >> 11) * (1.0 / 9007199254740992.0) * 2.0 - 1.0


def test_channel_velocity_generator(orc):
    nx, ny, nz, uc, amp, seed = 6, 5, 4, 0.05, 0.05, 99
    ux, uy, uz = orc.channel_velocity(nx, ny, nz, uc, amp, seed)
    for ix, iy, iz in [(0, 0, 0), (5, 4, 3), (2, 3, 1)]:
        lin = ix + nx * (iy + ny * iz)
        assert ux[ix, iy, iz] == amp * uc * numpy_uniform_pm1(seed, 3 * lin)
        xx0 = abs(ix + 0.5 - nx / 2)
        prof = (4.0 * uc) * ((nx / 2) ** 2 - xx0**2) / (nx * nx)
        assert uy[ix, iy, iz] == prof + amp * uc * numpy_uniform_pm1(seed, 3 * lin + 1)
    assert np.abs(ux).max() <= amp * uc and np.abs(uz).max() <= amp * uc


def test_loglaw_velocity_is_initvel_turbulent_start(orc):
    """initvel's ivel branch (initial.f90:101-147) by hand in numpy: the law
    of the wall (u+ = y+ below y+ = 10.8, ln(y+)/0.41 + 5 above), mirrored
    onto the upper half, the middle plane of an odd channel at rest, and the
    perturbation with A9 from the reference's formulas."""
    nx, ny, nz, ustar, visc = 41, 12, 10, 0.0035, 0.0012
    ystar = visc / ustar
    ux, uy, uz = orc.loglaw_velocity(nx, ny, nz, ustar, ystar, 0.0)
    assert not ux.any() and not uz.any()
    yp = (np.arange(1, nx // 2 + 1) - 0.5) / ystar
    prof = np.where(yp < 10.8, yp * ustar, (np.log(yp) / 0.41 + 5.0) * ustar)
    assert np.allclose(uy[: nx // 2, 3, 4], prof, rtol=1e-15, atol=0)
    assert np.array_equal(uy[::-1], uy)
    assert not uy[nx // 2].any()
    a9 = 1.5
    px, py, _ = orc.loglaw_velocity(nx, ny, nz, ustar, ystar, a9)
    pi2 = 2 * np.pi
    j, k = 5, 7
    arg = pi2 * (j + 1 - 0.5) / ny + pi2 * (k + 1 - 0.5) / nz
    e = np.exp(-yp / 60.0)
    ccc1 = -ny / pi2 / ystar * a9 * ustar / 60.0 / 60.0
    assert np.allclose(py[: nx // 2, j, k], prof + ccc1 * yp * e * np.sin(arg), rtol=1e-13, atol=0)
    assert np.allclose(px[: nx // 2, j, k], a9 * ustar * (1 - e - yp / 60.0 * e) * np.cos(arg), rtol=1e-12,
                       atol=1e-18)
    assert np.array_equal(px[::-1], px)


def test_oracle_reproduces_golden_fixture(orc):
    """The committed fixture (tests/golden/make_golden.py) pins the oracle."""
    import importlib.util
    from pathlib import Path
    here = Path(__file__).resolve().parent / "golden"
    spec = importlib.util.spec_from_file_location("make_golden", here / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    g = np.load(here / "channel_6x10x4.npz")
    assert np.array_equal(mg.initial_state(), g["f0"])
    p = orc.params(mg.rates(), mg.FORCE)
    for n in g["steps"]:
        f, rho, ux, uy, uz = orc.run(p, g["f0"], int(n), mode=0)
        assert np.array_equal(f, g[f"f{n}"])
        assert np.array_equal(np.stack([rho, ux, uy, uz]), g[f"macro{n}"])
