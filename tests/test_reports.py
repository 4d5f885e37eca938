"""Committed measurement reports: complete, and within the bars they are
quoted against.

precision_sweep_512x256x256_report.json is the output of
d3q19-single-phase_gb300/precision_sweep.py on one GB300 (the particle-laden
channel 512 x 256 x 256 with 2048 spheres of radius 8, 20000 steps, run in
FP64, FP32 and FP16 storage from the same seeded state).  The bar: FP32 and
FP16 storage within 1% of FP64 in the mean velocity profile and the Reynolds
shear stress, averaged over the second half of the run.
"""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

GOLDEN = Path(__file__).resolve().parent / "golden"


def test_precision_sweep_report():
    r = json.loads((GOLDEN / "precision_sweep_512x256x256_report.json").read_text())
    assert r["grid_stream_span_wall"] == [512, 256, 256] and r["spheres"] == 2048 and r["steps"] == 20000
    for p in ("fp64", "fp32", "fp16"):
        assert r["runs"][p]["fail"] is None and r["runs"][p]["steps_done"] == 20000
        assert len(r["series"][p]) == r["steps"] // r["every"]
    for p in ("fp32", "fp16"):
        e = r["errors"][p]
        assert e["mean_profile_rel_err"] < 0.01
        assert e["reynolds_stress_rel_err"] < 0.01
        assert e["drag_mean_rel_err"] < 0.01
    # FP64 keeps the fluid mass (the mean density is removed every 100 steps)
    assert abs(r["runs"]["fp64"]["mean_density_drift"]) < 1e-15
    # the averaged profiles in the report reproduce its error figures
    ref = np.array(r["profiles"]["fp64"]["mean"])
    lp = np.array(r["profiles"]["fp16"]["mean"])
    assert np.isclose(np.abs(lp - ref).max() / np.abs(ref).max(), r["errors"]["fp16"]["mean_profile_rel_err"])
