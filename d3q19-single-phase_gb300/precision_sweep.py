"""Precision sweep of the particle-laden channel on one GPU.

The same seeded run three ways -- FP64 storage and arithmetic, FP32 storage
and arithmetic, FP32 arithmetic on FP16-stored deviations f_i - w_i under a
fixed scale -- and the errors of the two lower precisions against FP64 in
the results the channel is run for: the mean streamwise velocity profile
u(z), the Reynolds shear stress <u'w'>(z) (wall-normal x streamwise), the
drag on the spheres and the drift of the fluid mass.

Default workload: 512 x 256 x 256 (streamwise x spanwise x wall-normal,
Re_tau ~ 181), 2048 spheres of radius 8 (density ratio 2) placed from a seed
with >= 2-node gaps and >= 1 node from the walls, the fluid started from the
equilibrium of the laminar Poiseuille profile plus seeded +-5% noise,
20000 steps.  Every `--every` steps each run records the plane statistics
(statistc2 normalisation), the spheres' forces and the fluid mass.  The
three runs start from bit-identical states, but the flow is chaotic: the
instantaneous fields drift apart at the rate rounding differences grow, so
the comparison is made on averages over the second half of the run (also
reported: the same errors on the last sample alone).

    python d3q19-single-phase_gb300/precision_sweep.py --out <dir> [--steps N] [--every K]
"""
from __future__ import annotations

import argparse
import importlib
import json
import sys
import time
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
if str(PKG_DIR.parent) not in sys.path:
    sys.path.insert(0, str(PKG_DIR.parent))
pkg = importlib.import_module(PKG_DIR.name)


def run_one(cfg, prec: str, pos, steps: int, every: int, device: int) -> dict:
    """One precision: samples every `every` steps (streamwise mean profile and
    Reynolds shear stress in wall units, mean and per-sphere streamwise drag,
    fluid mass), GPU seconds per step, and the step of a failure if any."""
    run = cfg.params(prec, device=device)
    samples = []
    fail = None
    t_steps = 0.0
    with pkg.Lattice(run) as lat:
        lat.init_channel(cfg.uc, cfg.amp, cfg.seed)
        lat.set_particles(pos, cfg.radius, 2.0)
        d0 = lat.diag()
        done = 0
        while done < steps:
            n = min(every, steps - done)
            t0 = time.perf_counter()
            try:
                lat.step(n)
            except pkg.LBMError as e:                 # runaway spheres, non-finite state
                fail = dict(step=done + n, error=str(e))
                break
            t_steps += time.perf_counter() - t0
            done += n
            d = lat.diag()
            if d.nonfinite:
                fail = dict(step=done, error="non-finite populations")
                break
            st = pkg.statistics(lat.profiles(), cfg.ustar)
            part = lat.particles()
            samples.append(dict(
                step=done,
                mean=st["mean"][:, 1].copy(),                  # <u_stream>/u*
                stress=st["stress"][:, 1].copy(),              # <u'_wall u'_stream>/u*^2
                drag=part["force"][:, 1].copy(),               # streamwise force per sphere
                rho_sum=d.rho_sum, nfluid=d.nfluid))
    return dict(precision=prec, samples=samples, fail=fail, d0_rho_sum=d0.rho_sum, d0_nfluid=d0.nfluid,
                s_per_step=t_steps / max(done, 1), steps_done=done)


def window(res: dict, lo: int) -> dict:
    """Averages over the samples with step > lo."""
    s = [x for x in res["samples"] if x["step"] > lo]
    if not s:
        return {}
    return dict(n=len(s), mean=np.mean([x["mean"] for x in s], 0), stress=np.mean([x["stress"] for x in s], 0),
                drag=float(np.mean([x["drag"].mean() for x in s])),
                drag_per_sphere=np.mean([x["drag"] for x in s], 0))


def rel_max(a, b) -> float:
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def compare(lp: dict, ref: dict, lo: int) -> dict:
    """Errors of one precision against FP64: time-averaged (steps > lo) and on
    the last common sample."""
    out = {}
    wa, wb = window(lp, lo), window(ref, lo)
    if wa and wb:
        out["window_samples"] = wa["n"]
        out["mean_profile_rel_err"] = rel_max(wa["mean"], wb["mean"])
        out["reynolds_stress_rel_err"] = rel_max(wa["stress"], wb["stress"])
        out["drag_mean_rel_err"] = abs(wa["drag"] - wb["drag"]) / max(abs(wb["drag"]), 1e-300)
        out["drag_per_sphere_rel_err"] = rel_max(wa["drag_per_sphere"], wb["drag_per_sphere"])
    common = min(len(lp["samples"]), len(ref["samples"]))
    if common:
        a, b = lp["samples"][common - 1], ref["samples"][common - 1]
        out["last_sample_step"] = a["step"]
        out["last_mean_profile_rel_err"] = rel_max(a["mean"], b["mean"])
        out["last_reynolds_stress_rel_err"] = rel_max(a["stress"], b["stress"])
        out["last_drag_mean_rel_err"] = abs(a["drag"].mean() - b["drag"].mean()) / max(abs(b["drag"].mean()), 1e-300)
    return out


def drift(res: dict) -> dict:
    """Fluid mass change and change of the mean density over the fluid nodes
    (the fluid node set changes as the spheres move) from the start."""
    if not res["samples"]:
        return {}
    last = res["samples"][-1]
    return dict(mass_drift=last["rho_sum"] - res["d0_rho_sum"],
                mean_density_drift=last["rho_sum"] / max(last["nfluid"], 1)
                - res["d0_rho_sum"] / max(res["d0_nfluid"], 1))


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--config", default="spheres-512x256x256", choices=sorted(pkg.CHANNEL_CONFIGS))
    ap.add_argument("--steps", type=int, default=None, help="default: the configuration's step count")
    ap.add_argument("--every", type=int, default=500)
    ap.add_argument("--precisions", default="fp64,fp32,fp16")
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--out", type=Path, required=True)
    args = ap.parse_args()
    cfg = pkg.CHANNEL_CONFIGS[args.config]
    if not cfg.spheres:
        raise SystemExit(f"{args.config} has no spheres")
    steps = args.steps or cfg.steps
    precs = args.precisions.split(",")
    if precs[0] != "fp64":
        raise SystemExit("the first precision must be fp64 (the reference of the comparison)")
    pos = pkg.place_spheres(cfg.wall, cfg.stream, cfg.span, cfg.spheres, cfg.radius, gap=2.0, wall_gap=1.0,
                            seed=cfg.seed)
    res = {}
    for p in precs:
        t0 = time.perf_counter()
        res[p] = run_one(cfg, p, pos, steps, args.every, args.device)
        print(f"[sweep] {p}: {res[p]['steps_done']} steps, {1e3 * res[p]['s_per_step']:.3f} ms/step, "
              f"fail={res[p]['fail']}, {time.perf_counter() - t0:.0f} s", flush=True)
    lo = steps // 2
    ref = res["fp64"]
    wref = window(ref, lo)
    report = dict(
        config=cfg.name, grid_stream_span_wall=[cfg.stream, cfg.span, cfg.wall], spheres=cfg.spheres,
        radius=cfg.radius, visc=cfg.visc, ustar=cfg.ustar, h=cfg.h, steps=steps, every=args.every,
        window=f"samples with step > {lo}", seed=cfg.seed,
        runs={p: dict(ms_per_step=1e3 * r["s_per_step"], steps_done=r["steps_done"], fail=r["fail"], **drift(r))
              for p, r in res.items()},
        fp64=dict(centreline_u_over_ustar=float(wref["mean"].max()) if wref else None,
                  peak_reynolds_stress=float(np.abs(wref["stress"]).max()) if wref else None,
                  mean_drag=wref.get("drag") if wref else None),
        errors={p: compare(res[p], ref, lo) for p in precs[1:]},
        profiles={p: dict(mean=window(r, lo)["mean"].tolist(), stress=window(r, lo)["stress"].tolist())
                  for p, r in res.items() if window(r, lo)},
        series={p: [dict(step=x["step"], drag=float(x["drag"].mean()), rho_sum=x["rho_sum"],
                         centreline=float(x["mean"].max()), peak_stress=float(np.abs(x["stress"]).max()))
                    for x in r["samples"]] for p, r in res.items()},
    )
    args.out.mkdir(parents=True, exist_ok=True)
    path = args.out / f"precision_sweep_{cfg.stream}x{cfg.span}x{cfg.wall}.json"
    path.write_text(json.dumps(report, indent=1))
    print(json.dumps(dict(runs=report["runs"], errors=report["errors"], fp64=report["fp64"]), indent=1))
    print(f"[sweep] report: {path}")


if __name__ == "__main__":
    main()
