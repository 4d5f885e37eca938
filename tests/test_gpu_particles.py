"""GPU moving-sphere kernels (interpolated bounce-back, momentum exchange,
Newton-Euler, refilling) through the C ABI against the FP64 oracle.

Tolerances: FP64 storage -- relative L-inf <= 1e-10 in the populations and in
particle positions, velocities, forces and torques (the parity bar for
particle forces); FP32/FP16 storage -- stability and forces within a few
percent of FP64.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def channel_with_spheres(orc, pkg, shape, pos, vel=None, seed=3, force=2e-6, precision="fp64"):
    nx, ny, nz = shape
    run = pkg.RunParams(nx=nx, ny=ny, nz=nz, visc=0.02, force_y=force, mrt_type=1,
                        precision=pkg.PRECISIONS[precision])
    u = orc.channel_velocity(nx, ny, nz, 0.04, 0.05, seed)
    f0 = orc.initpop(*u)
    return run, f0


POS = np.array([[8.3, 10.2, 7.7], [15.6, 21.9, 13.1], [12.0, 4.4, 16.8]])
VEL = np.array([[0.0, 0.01, 0.0], [0.002, -0.003, 0.001], [0.0, 0.0, 0.004]])


@pytest.mark.parametrize("nsteps", [1, 2, 25])
def test_particles_fp64_match_oracle(pkg, orc, nsteps):
    shape = (24, 32, 22)
    run, f0 = channel_with_spheres(orc, pkg, shape, POS)
    sp = orc.Spheres(POS, radius=4.0, rho_ratio=2.0, vel=VEL)
    fo, owner, links, refills = orc.particle_run(orc.params_from(run), sp, f0, nsteps)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f0)
        lat.set_particles(POS, radius=4.0, rho_ratio=2.0, vel=VEL)
        lat.step(nsteps)
        g = lat.download_f()
        st = lat.particles()
        nsolid, nlinks, nref = lat.particle_counts()
    assert nlinks == links[-1]
    assert nref == refills[-1]
    assert nsolid == int((owner >= 0).sum())
    assert rel(g, fo) < 1e-10
    for k in ("pos", "vel", "omg", "force", "torque"):
        assert rel(st[k], getattr(sp, k)) < 1e-10, k


def test_large_sphere_64bit_rows_match_oracle(pkg, orc):
    """Radius 12: the staged rows of the bounce-back kernel exceed 32 nodes and
    take 64-bit words."""
    shape = (32, 40, 40)
    pos = np.array([[16.2, 19.7, 20.4]])
    vel = np.array([[0.001, 0.004, -0.002]])
    run, f0 = channel_with_spheres(orc, pkg, shape, pos)
    sp = orc.Spheres(pos, radius=12.0, rho_ratio=2.0, vel=vel)
    fo, owner, links, refills = orc.particle_run(orc.params_from(run), sp, f0, 3)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f0)
        lat.set_particles(pos, radius=12.0, rho_ratio=2.0, vel=vel)
        lat.step(3)
        g = lat.download_f()
        st = lat.particles()
        _, nlinks, nref = lat.particle_counts()
    assert nlinks == links[-1] and nref == refills[-1]
    assert rel(g, fo) < 1e-10
    for k in ("pos", "vel", "omg", "force", "torque"):
        assert rel(st[k], getattr(sp, k)) < 1e-10, k


def test_repulsion_cell_list_matches_oracle(pkg, orc):
    """Spheres in contact (one pair across the periodic streamwise boundary,
    one near a wall): the cell-list repulsion gives the oracle's
    index-ordered all-pairs sum."""
    shape = (24, 48, 40)
    pos = np.array([[12.0, 10.0, 10.0], [12.3, 18.6, 10.2], [6.0, 3.0, 30.0], [6.4, 42.6, 30.5],
                    [4.6, 30.0, 20.0], [17.0, 30.0, 31.0]])
    run, f0 = channel_with_spheres(orc, pkg, shape, pos)
    sp = orc.Spheres(pos, radius=4.0, rho_ratio=2.0)
    fo, owner, links, refills = orc.particle_run(orc.params_from(run), sp, f0, 4)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f0)
        lat.set_particles(pos, radius=4.0, rho_ratio=2.0)
        lat.step(4)
        g = lat.download_f()
        st = lat.particles()
    assert rel(g, fo) < 1e-10
    for k in ("pos", "vel", "omg", "force", "torque"):
        assert rel(st[k], getattr(sp, k)) < 1e-10, k
    # the contacts matter: without repulsion the spheres of the pairs move otherwise
    free = orc.Spheres(pos, radius=4.0, rho_ratio=2.0, stf0=0.0, stf1=0.0, stf0_w=0.0, stf1_w=0.0)
    orc.particle_run(orc.params_from(run), free, f0, 4)
    assert rel(free.vel[:5], sp.vel[:5]) > 1e-3


def test_overlapping_spheres_ownership_matches_oracle(pkg, orc):
    """Two overlapping spheres driven apart: nodes in the overlap belong to the
    higher index, and the nodes that sphere 1 leaves inside sphere 0 are
    claimed by sphere 0 (the oracle claims every inside node in index
    order)."""
    shape = (24, 48, 40)
    pos = np.array([[12.0, 20.0, 20.0], [12.3, 25.0, 20.5], [12.0, 38.0, 8.0]])
    vel = np.array([[0.0, -0.06, 0.0], [0.0, 0.06, 0.0], [0.0, 0.0, 0.0]])
    run, f0 = channel_with_spheres(orc, pkg, shape, pos)
    sp = orc.Spheres(pos, radius=4.0, rho_ratio=1e6, vel=vel)
    fo, owner, links, refills = orc.particle_run(orc.params_from(run), sp, f0, 30)
    assert sum(refills) > 0
    with pkg.Lattice(run) as lat:
        lat.upload_f(f0)
        lat.set_particles(pos, radius=4.0, rho_ratio=1e6, vel=vel)
        lat.step(30)
        g = lat.download_f()
        st = lat.particles()
        nsolid, nlinks, _ = lat.particle_counts()
        rho, _, _, _ = lat.macrovar()
    assert nsolid == int((owner >= 0).sum()) and nlinks == links[-1]
    assert rel(g, fo) < 1e-10
    for k in ("pos", "vel", "omg", "force", "torque"):
        assert rel(st[k], getattr(sp, k)) < 1e-10, k


@pytest.mark.parametrize("prec", ["fp32", "fp16"])
def test_fp64_link_fractions_option(pkg, orc, prec):
    """LBM_PFLAG_Q_FP64: the FP32 link fractions (exact integer offsets plus an
    FP32 fraction) and FP64 ones give the same run to within the storage
    rounding, and both follow the FP64 path."""
    shape = (32, 64, 32)
    pos = pkg.place_spheres(*shape, 6, 4.0, gap=2.0, wall_gap=1.0, seed=13)
    res = {}
    for tag, p, flags in (("ref", "fp64", 0), ("q32", prec, 0), ("q64", prec, pkg.PFLAG_Q_FP64)):
        run, f0 = channel_with_spheres(orc, pkg, shape, pos, force=1e-5, precision=p)
        with pkg.Lattice(run) as lat:
            lat.upload_f(f0)
            lat.set_particles(pos, radius=4.0, rho_ratio=2.0, flags=flags)
            lat.step(40)
            res[tag] = lat.particles()
    tol = 1e-4 if prec == "fp32" else 3e-2
    for tag in ("q32", "q64"):
        assert rel(res[tag]["force"], res["ref"]["force"]) < tol, tag
    assert rel(res["q32"]["force"], res["q64"]["force"]) < tol


def test_particle_diagnostics_mask_solid_nodes(pkg, orc):
    shape = (24, 32, 22)
    run, f0 = channel_with_spheres(orc, pkg, shape, POS)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f0)
        lat.set_particles(POS, radius=4.0, rho_ratio=2.0)
        lat.step(3)
        nsolid, _, _ = lat.particle_counts()
        st = lat.diag()
        rho, ux, uy, uz = lat.macrovar()
        prof = lat.profiles()
        pst = lat.particles()
    assert st.nfluid == np.prod(shape) - nsolid
    solid = rho == 2.0                                   # rho = rhopart on solid nodes (macrovar)
    assert solid.sum() == nsolid
    assert prof[:, 11].sum() == st.nfluid
    # solid nodes carry the rigid-body velocity of their sphere
    ix, iy, iz = np.argwhere(solid)[0]
    d = np.array([ix + 0.5, iy + 0.5, iz + 0.5]) - pst["pos"]
    d[:, 1] = (d[:, 1] + shape[1] / 2) % shape[1] - shape[1] / 2
    d[:, 2] = (d[:, 2] + shape[2] / 2) % shape[2] - shape[2] / 2
    k = int(np.argmin((d**2).sum(1)))
    want = pst["vel"][k] + np.cross(pst["omg"][k], d[k])
    np.testing.assert_allclose([ux[ix, iy, iz], uy[ix, iy, iz], uz[ix, iy, iz]], want, rtol=1e-12, atol=1e-15)


def test_sphere_placement(pkg):
    nx, ny, nz, n, R = 64, 128, 128, 256, 4.0
    pos = pkg.place_spheres(nx, ny, nz, n, R, gap=2.0, wall_gap=1.0, seed=7)
    again = pkg.place_spheres(nx, ny, nz, n, R, gap=2.0, wall_gap=1.0, seed=7)
    assert np.array_equal(pos, again)
    assert (pos[:, 0] - R >= 1.0).all() and (pos[:, 0] + R <= nx - 1.0).all()
    d = pos[:, None, :] - pos[None, :, :]
    d[..., 1] = (d[..., 1] + ny / 2) % ny - ny / 2
    d[..., 2] = (d[..., 2] + nz / 2) % nz - nz / 2
    dist = np.sqrt((d**2).sum(-1)) + np.eye(n) * 1e9
    assert dist.min() >= 2 * R + 2.0


@pytest.mark.parametrize("prec", ["fp32", "fp16"])
def test_particles_low_precision_follow_fp64(pkg, orc, prec):
    shape = (32, 64, 32)
    pos = pkg.place_spheres(*shape, 6, 4.0, gap=2.0, wall_gap=1.0, seed=11)
    res = {}
    for p in ("fp64", prec):
        run, f0 = channel_with_spheres(orc, pkg, shape, pos, force=1e-5, precision=p)
        with pkg.Lattice(run) as lat:
            lat.upload_f(f0)
            lat.set_particles(pos, radius=4.0, rho_ratio=2.0)
            lat.step(60)
            res[p] = (lat.particles(), lat.diag())
    a, b = res[prec][0], res["fp64"][0]
    assert res[prec][1].nonfinite == 0
    assert rel(a["vel"], b["vel"]) < (1e-4 if prec == "fp32" else 3e-2)
    assert rel(a["pos"], b["pos"]) < 1e-6


def test_mean_density_removed_every_100_steps_with_spheres(pkg, orc):
    """main.f90:163-167: with particles the mean fluid density is removed
    every 100 steps (avedensity), so after step 100 it is zero again."""
    shape = (24, 32, 22)
    run, f0 = channel_with_spheres(orc, pkg, shape, POS)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f0)
        lat.set_particles(POS, radius=4.0, rho_ratio=2.0, vel=VEL)
        lat.step(99)
        d99 = lat.diag()
        lat.step(1)
        d100 = lat.diag()
    assert abs(d99.rho_sum / d99.nfluid) > 1e-9
    assert abs(d100.rho_sum / d100.nfluid) < 1e-13


def test_mean_density_removed_at_odd_parity(pkg, orc):
    """A run continued from step 1 reaches step 100 after an odd number of
    steps (array in the parity-1 layout); the removal still happens at step
    100, as main.f90:163 counts absolute steps."""
    shape = (24, 32, 22)
    run, f0 = channel_with_spheres(orc, pkg, shape, POS)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f0)
        lat.set_particles(POS, radius=4.0, rho_ratio=2.0, vel=VEL)
        lat.set_step_count(1)
        lat.step(98)
        d99 = lat.diag()
        lat.step(1)
        d100 = lat.diag()
        assert lat.step_count() == 100
    assert abs(d99.rho_sum / d99.nfluid) > 1e-9
    assert abs(d100.rho_sum / d100.nfluid) < 1e-13


def test_step_launch_count(pkg, orc):
    """lbm_step_launches counts the kernels the steps launch: one per fluid
    step, the sphere pass after each step, the two kernels of the
    mean-density removal at every step number that is a multiple of 100, and
    the three of the spheres' spatial re-sort every 100 steps."""
    shape = (24, 32, 22)
    run, f0 = channel_with_spheres(orc, pkg, shape, POS)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f0)
        n0 = lat.step_launches()
        lat.step(3)
        assert lat.step_launches() - n0 == 3          # fluid only
        lat.set_particles(POS, radius=4.0, rho_ratio=2.0, vel=VEL)
        n1, s1 = lat.step_launches(), lat.step_count()
        lat.step(110)
        removals = sum(1 for k in range(s1 + 1, s1 + 111) if k % 100 == 0)
        resorts = 110 // 100                           # the spatial order, every 100 steps after set
        per = (lat.step_launches() - n1 - 2 * removals - 3 * resorts) / 110
        assert per in (9.0, 10.0)                      # 1 fluid + 8 or 9 sphere kernels


def test_config1_fp64_matches_oracle(pkg, orc):
    """The particle-laden channel at full size (256 x 128 x 128, 256 spheres of
    radius 4, density ratio 2, seeded placement and initial state), FP64:
    populations and sphere state within 1e-10 of the oracle after 10 steps,
    link and refill counts equal."""
    cfg = pkg.CHANNEL_CONFIGS["spheres-256x128x128"]
    run = cfg.params("fp64")
    pos = pkg.place_spheres(cfg.wall, cfg.stream, cfg.span, cfg.spheres, cfg.radius, gap=2.0, wall_gap=1.0,
                            seed=cfg.seed)
    u = orc.channel_velocity(run.nx, run.ny, run.nz, cfg.uc, cfg.amp, cfg.seed)
    f0 = orc.initpop(*u)
    sp = orc.Spheres(pos, radius=cfg.radius, rho_ratio=2.0)
    fo, owner, links, refills = orc.particle_run(orc.params_from(run), sp, f0, 10)
    with pkg.Lattice(run) as lat:
        lat.init_channel(cfg.uc, cfg.amp, cfg.seed)
        assert np.array_equal(lat.download_f(), f0)
        lat.set_particles(pos, cfg.radius, 2.0)
        lat.step(10)
        g = lat.download_f()
        st = lat.particles()
        nsolid, nlinks, nref = lat.particle_counts()
    assert nlinks == links[-1] and nref == refills[-1]
    assert nsolid == int((owner >= 0).sum())
    assert rel(g, fo) < 1e-10
    for k in ("pos", "vel", "omg", "force", "torque"):
        assert rel(st[k], getattr(sp, k)) < 1e-10, k


def test_particles_fp64_match_oracle_across_resort(pkg, orc):
    """106 steps: the bounce-back kernel's spatial order of the spheres is
    re-sorted from their positions at step 100 (the order in which CTAs take
    the spheres, which changes no result) and the mean fluid density is
    removed after step 100 (applied to the oracle's state here as the
    library applies it: w_i times the mean over fluid nodes off every
    population).  Populations and sphere state stay within 1e-10."""
    shape = (24, 32, 22)
    run, f0 = channel_with_spheres(orc, pkg, shape, POS)
    p = orc.params_from(run)
    sp = orc.Spheres(POS, radius=4.0, rho_ratio=2.0, vel=VEL)
    fo, owner, _, _ = orc.particle_run(p, sp, f0, 100)
    fluid = owner < 0
    mean = fo[:, fluid].sum() / fluid.sum()
    fo = fo - (orc.W * mean)[:, None, None, None]
    fo, owner, links, _ = orc.particle_run(p, sp, fo, 6, owner=owner)
    with pkg.Lattice(run) as lat:
        lat.upload_f(f0)
        lat.set_particles(POS, radius=4.0, rho_ratio=2.0, vel=VEL)
        lat.step(106)
        g = lat.download_f()
        st = lat.particles()
        assert lat.particle_counts()[1] == links[-1]
    assert rel(g, fo) < 1e-10
    for k in ("pos", "vel", "omg", "force", "torque"):
        assert rel(st[k], getattr(sp, k)) < 1e-10, k
