"""CPU checks of the oracle's strain rate (sijstat01's two methods): both give
the analytic S_ij S_ij of a laminar Poiseuille flow, and agree with each
other on a developed channel; dissipation_calc's plane statistics give the
analytic shear S_xy."""
from __future__ import annotations

import numpy as np

from test_oracle import stable_rates


def test_poiseuille_strain_both_methods(orc):
    nx, ny, nz = 16, 4, 4
    visc, g = 0.1, 1e-5
    rates = stable_rates(visc)
    p = orc.params(rates, (0.0, g, 0.0))
    zero = np.zeros((nx, ny, nz), order="F")
    f = orc.initpop(zero, zero, zero)
    f = orc.run(p, f, 4000)[0]
    m1, m2 = orc.strain_sij2(p, f, rates["s1"], rates["s9"])
    x = np.arange(nx) + 0.5                   # node centres, walls at 0 and nx
    dudx = g / (2 * visc) * (nx - 2 * x)      # u = g x (nx - x) / (2 visc)
    exact = 0.5 * dudx**2                     # S_xy = S_yx = du/dx / 2
    for m in (m1, m2):
        prof = m.mean(axis=(1, 2))
        assert np.abs(prof - exact).max() < 2e-2 * exact.max()
    assert np.abs(m1 - m2).max() < 2e-2 * exact.max()
    # dissipation_calc's plane means: the same S_ij S_ij, and its two S_xy
    # columns as the reference writes them: method 1 (-1.5 neqm13) gives
    # +du/dx / 2, method 2 ((1.5 / tau) sum f_neq c_x c_y, with Chapman-Enskog
    # sum f_neq c_x c_y = -(2 tau / 3) S_xy) gives -du/dx / 2
    d = orc.dissipation_sums(p, f, rates["s1"], rates["s9"])
    assert (d[:, 4] == ny * nz).all()
    assert np.allclose(d[:, 0] / d[:, 4], m1.mean(axis=(1, 2)), rtol=1e-12, atol=0)
    assert np.allclose(d[:, 1] / d[:, 4], m2.mean(axis=(1, 2)), rtol=1e-12, atol=0)
    for k, sign in ((2, 1.0), (3, -1.0)):
        assert np.abs(d[:, k] / d[:, 4] - sign * 0.5 * dudx).max() < 2e-2 * np.abs(0.5 * dudx).max()
    solid = np.zeros((nx, ny, nz), dtype=bool)
    solid[3, 1, 2] = True
    ds = orc.dissipation_sums(p, f, rates["s1"], rates["s9"], solid)
    assert ds[3, 4] == ny * nz - 1 and np.isclose(ds[3, 0], d[3, 0] - m1[3, 1, 2], rtol=1e-12)


def test_strain_zero_at_equilibrium(orc):
    rng = np.random.default_rng(1)
    shape = (6, 5, 4)
    u = [rng.uniform(-0.02, 0.02, shape) for _ in range(3)]
    f = orc.initpop(*u)
    p = orc.params(stable_rates(0.05))
    m1, m2 = orc.strain_sij2(p, f, 1.5, 1.2)
    # equilibrium populations carry no non-equilibrium part (up to the F/2 of
    # a zero force) -- both measures vanish to rounding
    assert np.abs(m1).max() < 1e-24 and np.abs(m2).max() < 1e-24


def test_laminar_flow_has_no_subgrid_viscosity(orc):
    """Box filtering a flow that varies only across the channel leaves a
    subgrid stress with no shear component, so the target eddy viscosity of
    the closure is zero."""
    nx, ny, nz = 16, 8, 8
    visc, g = 0.1, 1e-5
    p = orc.params(stable_rates(visc), (0.0, g, 0.0))
    zero = np.zeros((nx, ny, nz), order="F")
    f = orc.run(p, orc.initpop(zero, zero, zero), 3000)[0]
    X, y, ub = orc.closure_training_data(p, f, 4, 0.005, 8.0)
    assert X.shape == (4 * 2 * 2, 7) and np.isfinite(X).all()
    assert np.abs(y).max() < 1e-10
    assert np.abs(ub[1]).max() > 0.01 * g / visc
