"""CPU checks of the oracle's moving-sphere algorithms (interpolated
bounce-back, momentum exchange, refilling, Newton-Euler).  The reference ships
no particle algorithm (it declares the data only), so these pin physics:
link geometry, drag direction and symmetry, momentum balance, stability of a
moving sphere, and agreement with the Stokes drag trend."""
from __future__ import annotations

import numpy as np
import pytest

from test_oracle import stable_rates


def lbgk(visc):
    s9 = 1.0 / (3 * visc + 0.5)
    return dict(s1=s9, s2=s9, s4=s9, s9=s9, s10=s9, s13=s9, s16=s9, omegepsl=3.0, omegepslj=-5.5, omegxx=-0.5)


def uniform_state(orc, shape, u):
    ux = np.full(shape, u[0], order="F")
    uy = np.full(shape, u[1], order="F")
    uz = np.full(shape, u[2], order="F")
    return orc.initpop(ux, uy, uz)


def test_solid_marking_and_link_geometry(orc):
    shape = (20, 24, 22)
    sp = orc.Spheres([[10.0, 12.3, 11.1]], radius=4.0)
    owner = orc.mark_solid(sp, shape)
    ix, iy, iz = np.nonzero(owner == 0)
    d = np.sqrt((ix + 0.5 - 10.0) ** 2 + (iy + 0.5 - 12.3) ** 2 + (iz + 0.5 - 11.1) ** 2)
    assert d.max() <= 4.0
    assert abs(len(ix) - 4 / 3 * np.pi * 4.0**3) < 0.1 * 4 / 3 * np.pi * 4.0**3
    p = orc.params(lbgk(0.1))
    f = uniform_state(orc, shape, (0.0, 0.0, 0.0))
    _, _, links, _ = orc.particle_run(p, sp, f, 1, owner=owner.copy())
    # about 5 links per unit surface (the estimate of para.f90:377)
    assert 0.5 * 5 * 4 * np.pi * 16 < links[0] < 2.0 * 5 * 4 * np.pi * 16


def test_fixed_sphere_in_uniform_flow_feels_drag_along_flow(orc):
    shape = (24, 24, 24)
    sp = orc.Spheres([[12.0, 12.0, 12.0]], radius=4.0, rho_ratio=1e12)   # effectively fixed
    p = orc.params(lbgk(0.1))
    f = uniform_state(orc, shape, (0.0, 0.02, 0.0))
    f, owner, links, _ = orc.particle_run(p, sp, f, 60)
    F = sp.force[0]
    assert F[1] > 0                                   # drag along the streamwise flow
    assert abs(F[0]) < 0.05 * F[1] and abs(F[2]) < 0.05 * F[1]   # symmetric sphere, centred
    assert np.abs(sp.torque[0]).max() < 0.05 * F[1] * 4.0


def test_momentum_balance_with_body_force(orc):
    """Fluid + sphere momentum grows by the body force acting on the whole
    volume (no walls in y/z; x walls take no streamwise momentum for a flow
    started from rest in the first steps)."""
    shape = (16, 16, 16)
    g = 1e-5
    p = orc.params(lbgk(0.1), (0.0, g, 0.0))
    sp = orc.Spheres([[8.0, 8.0, 8.0]], radius=3.0, rho_ratio=2.0)
    f = uniform_state(orc, shape, (0.0, 0.0, 0.0))
    steps = 3
    f, owner, _, _ = orc.particle_run(p, sp, f, steps)
    fluid = owner == -1
    jy = (orc.CY[:, None, None, None] * f).sum(axis=0)
    vol = 4 / 3 * np.pi * 27.0
    m = 2.0 * vol
    total = jy[fluid].sum() + m * sp.vel[0, 1]
    expect = g * steps * (fluid.sum() + vol)
    assert total == pytest.approx(expect, rel=0.1)


def test_moving_sphere_refills_and_stays_finite(orc):
    shape = (20, 40, 20)
    sp = orc.Spheres([[10.0, 12.0, 10.0]], radius=4.0, rho_ratio=1e12, vel=[[0.0, 0.05, 0.0]])
    p = orc.params(stable_rates(0.02))
    f = uniform_state(orc, shape, (0.0, 0.0, 0.0))
    f, owner, links, refills = orc.particle_run(p, sp, f, 100)
    assert np.isfinite(f).all()
    assert sum(refills) > 0
    assert sp.pos[0, 1] == pytest.approx(12.0 + 100 * 0.05, rel=1e-9)
    assert (owner == 0).sum() == pytest.approx(4 / 3 * np.pi * 64, rel=0.1)
    # the sphere drags fluid along
    uy = (orc.CY[:, None, None, None] * f).sum(axis=0)
    assert uy[owner == -1].sum() > 0


def test_drag_grows_linearly_with_velocity(orc):
    """Stokes regime: drag is proportional to the slip velocity."""
    shape = (24, 24, 24)
    p = orc.params(lbgk(0.1))
    drags = []
    for u in (0.002, 0.004):
        sp = orc.Spheres([[12.0, 12.0, 12.0]], radius=4.0, rho_ratio=1e12)
        f = uniform_state(orc, shape, (0.0, u, 0.0))
        orc.particle_run(p, sp, f, 80)
        drags.append(sp.force[0, 1])
    assert drags[1] / drags[0] == pytest.approx(2.0, rel=0.02)


def test_repulsion_pushes_touching_spheres_apart(orc):
    shape = (30, 40, 30)
    p = orc.params(lbgk(0.1))
    sp = orc.Spheres([[15.0, 15.0, 15.0], [15.0, 23.6, 15.0]], radius=4.0, rho_ratio=2.0)
    f = uniform_state(orc, shape, (0.0, 0.0, 0.0))
    orc.particle_run(p, sp, f, 5)
    assert sp.vel[0, 1] < 0 < sp.vel[1, 1]
