"""Committed measurement reports: complete, and within the bars they are
quoted against.

precision_sweep_<grid>_report.json is the output of
d3q19-single-phase_gb300/precision_sweep.py on one GB300: a particle-laden
channel run in FP64, FP32 and FP16 storage from the same seeded state --
512 x 256 x 256 with 2048 spheres of radius 8 for 20000 steps, and
256 x 128 x 128 with 256 spheres of radius 4 for 5000 steps.  The bar: FP32
and FP16 storage within 1% of FP64 in the mean velocity profile, the
Reynolds shear stress and the mean sphere drag, averaged over the second
half of the run.  The runs use MRTtype 1's rates (s16 = 1.98) and the
bounce-back of the library (quadratic for q < 1/2, linear for q >= 1/2).
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


@pytest.mark.parametrize("grid,shape,spheres,steps,fp16_drag", [
    ("512x256x256", [512, 256, 256], 2048, 20000, 0.01),
    ("256x128x128", [256, 128, 128], 256, 5000, 0.01),
])
def test_precision_sweep_report(grid, shape, spheres, steps, fp16_drag):
    r = json.loads((GOLDEN / f"precision_sweep_{grid}_report.json").read_text())
    assert r["grid_stream_span_wall"] == shape and r["spheres"] == spheres and r["steps"] == steps
    for p in ("fp64", "fp32", "fp16"):
        assert r["runs"][p]["fail"] is None and r["runs"][p]["steps_done"] == steps
        assert len(r["series"][p]) == r["steps"] // r["every"]
    for p in ("fp32", "fp16"):
        e = r["errors"][p]
        assert e["mean_profile_rel_err"] < 0.01
        assert e["reynolds_stress_rel_err"] < 0.01
    assert r["errors"]["fp32"]["drag_mean_rel_err"] < 0.01
    assert r["errors"]["fp16"]["drag_mean_rel_err"] < fp16_drag
    # FP64 keeps the fluid mass (the mean density is removed every 100 steps)
    assert abs(r["runs"]["fp64"]["mean_density_drift"]) < 1e-15
    # the averaged profiles in the report reproduce its error figures
    ref = np.array(r["profiles"]["fp64"]["mean"])
    lp = np.array(r["profiles"]["fp16"]["mean"])
    assert np.isclose(np.abs(lp - ref).max() / np.abs(ref).max(), r["errors"]["fp16"]["mean_profile_rel_err"])


def test_precision_sweep_from_developed_turbulence():
    """The same comparison from developed turbulence (precision_sweep.py
    --start developed): a particle-free FP32 DNS of the 512 x 256 x 256
    channel is run 200000 steps from a streak/vortex trigger, its populations
    start all runs, the 2048 spheres are added and every run covers 6000
    steps.  The FP64 Reynolds shear stress peaks at ~0.9 u*^2 in the window
    (0.75 at the end of the spin-up).  FP32 and FP16 storage stay within 1%
    of FP64 in the mean profile, the Reynolds stress and the mean drag; the
    chaos floor (a second FP64 run from populations perturbed by 1e-12) is
    far below, so the FP16 figures are precision errors, not decorrelation.
    All runs share the mean-density change of the first removal (the DNS
    state's mean density over the fluid nodes, -1.8e-7)."""
    r = json.loads((GOLDEN / "precision_sweep_512x256x256_developed_report.json").read_text())
    assert r["start"] == "developed" and r["spinup"]["steps"] == 200000
    assert r["spinup"]["history"][-1][1] >= 0.6
    assert max(x["peak_stress"] for x in r["series"]["fp64"]) >= 0.6
    for p in ("fp64", "fp64_perturbed", "fp32", "fp16"):
        assert r["runs"][p]["fail"] is None and r["runs"][p]["steps_done"] == r["steps"] == 6000
    for p in ("fp32", "fp16"):
        e = r["errors"][p]
        assert e["mean_profile_rel_err"] < 0.01 and e["reynolds_stress_rel_err"] < 0.01
        assert e["drag_mean_rel_err"] < 0.01
    floor = r["errors"]["fp64_perturbed"]
    assert floor["reynolds_stress_rel_err"] < 1e-5 < r["errors"]["fp16"]["reynolds_stress_rel_err"]
    d64, d32 = r["runs"]["fp64"]["mean_density_drift"], r["runs"]["fp32"]["mean_density_drift"]
    assert abs(d64 - d32) < 1e-9


def test_closure_a_posteriori_report():
    """The learned closure a posteriori (les_closure.py --window 400000): the
    coarse 128 x 64 x 64 LES (filter 4) and the 64 x 32 x 32 LES (filter 8),
    each with the closure, with the closure damped near the walls (van Driest,
    A+ = 26) and as plain under-resolved MRT, all from the last filtered
    snapshot over the DNS's continued window; mean streamwise profiles
    averaged over the second half against the box-averaged DNS.  At filter 4
    the wall-damped closure lowers the largest deviation from the DNS below
    that of plain MRT by more than a point, at >= 20x less GPU time than the
    DNS; at filter 8 the closure over-damps the coarse wall cells and plain
    MRT stays better."""
    r = json.loads((GOLDEN / "closure_channel_512x256x256_report.json").read_text())
    f4, f8 = r["factors"]["4"], r["factors"]["8"]
    err = {k: v["mean_profile_rel_err"] for k, v in f4["les"].items()}
    assert all(v["failed_at_step"] is None for f in (f4, f8) for v in f["les"].values())
    assert err["closure_wall_damped"] < err["plain_mrt"] - 0.01
    assert err["closure_wall_damped"] < 0.035
    assert f4["gpu_time_ratio_dns_over_les"] >= 20.0
    assert f8["les"]["plain_mrt"]["mean_profile_rel_err"] < f8["les"]["closure"]["mean_profile_rel_err"]
    # the damping acts at the wall and leaves the core
    nd, nu = f4["les"]["closure_wall_damped"]["nut_over_nu_profile"], f4["les"]["closure"]["nut_over_nu_profile"]
    assert nd[0] < 0.05 * nu[0] and nd[len(nd) // 2] > 0.5 * nu[len(nu) // 2]


def _sweep_module():
    import importlib.util
    path = Path(__file__).resolve().parents[1] / "d3q19-single-phase_gb300" / "precision_sweep.py"
    spec = importlib.util.spec_from_file_location("precision_sweep", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _fake_run(scale, steps=(500, 1000, 1500, 2000), drag=None):
    z = np.linspace(0.0, 1.0, 16)
    return dict(samples=[dict(step=s, mean=scale * 18 * z * (2 - z), stress=scale * np.sin(3 * z),
                              drag=(np.full(4, 1e-3) if drag is None else drag) * scale,
                              rho_sum=1e-3 * s, nfluid=1000) for s in steps],
                d0_rho_sum=0.0, d0_nfluid=1000, fail=None, s_per_step=1e-3, steps_done=steps[-1])


def test_sweep_errors_and_drift():
    """precision_sweep.py: errors are taken on the averages over the samples
    after the window start, relative to the FP64 maximum, and the drifts
    from the initial fluid mass."""
    ps = _sweep_module()
    ref, lp = _fake_run(1.0), _fake_run(1.02)
    e = ps.compare(lp, ref, 1000)
    assert e["window_samples"] == 2 and e["last_sample_step"] == 2000
    for k in ("mean_profile_rel_err", "reynolds_stress_rel_err", "drag_mean_rel_err", "last_mean_profile_rel_err"):
        assert e[k] == pytest.approx(0.02, rel=1e-9)
    d = ps.drift(ref)
    assert d["mass_drift"] == pytest.approx(2.0) and d["mean_density_drift"] == pytest.approx(2e-3)
    assert ps.window(ref, 5000) == {}                     # no sample after the window start
