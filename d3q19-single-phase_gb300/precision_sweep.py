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

--start developed: the runs start instead from developed turbulence.  A
particle-free FP32 DNS of the same channel is driven from a streak/vortex
trigger for --spinup steps (the Reynolds shear stress then peaks at
0.6-0.9 u*^2); its populations are copied into each precision's lattice
(FP16 storage rounds them once), the spheres are placed, and every run
covers the same --steps window.  In developed turbulence the three
trajectories decorrelate within the window whatever the precision, so the
report also carries the chaos floor: a second FP64 run from the same state
with relative perturbations of 1e-12 in the populations, compared with the
first FP64 run the same way.  A precision whose errors sit at that floor is
indistinguishable from FP64 in the statistics the window can resolve.
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


def run_one(cfg, prec: str, pos, steps: int, every: int, device: int, f0=None) -> dict:
    """One precision: samples every `every` steps (streamwise mean profile and
    Reynolds shear stress in wall units, mean and per-sphere streamwise drag,
    fluid mass), GPU seconds per step, and the step of a failure if any.
    f0: initial populations (reference layout); default the seeded
    Poiseuille start."""
    run = cfg.params(prec, device=device)
    samples = []
    fail = None
    t_steps = 0.0
    with pkg.Lattice(run) as lat:
        if f0 is None:
            lat.init_channel(cfg.uc, cfg.amp, cfg.seed)
        else:
            lat.upload_f(f0)
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


def trigger_velocity(nx, ny, nz, h, u0, amp, seed):
    """Initial velocity that becomes turbulent (reference axes, x wall-normal):
    a parabolic mean profile with centreline u0, streamwise vortices and
    streaks of spanwise wavelength nz/4 and seeded uniform noise of
    +-amp*u0."""
    eta = (np.arange(nx) + 0.5) / h - 1.0
    E, Y, Z = np.meshgrid(eta, np.arange(ny), np.arange(nz), indexing="ij")
    beta = 2 * np.pi * 4 / nz
    alpha = 2 * np.pi * 2 / ny
    a = 0.15 * u0
    ux = a * (1 - E**2) ** 2 * np.cos(beta * Z) * (1 + 0.3 * np.sin(alpha * Y))
    uz = 4 * a * E * (1 - E**2) * np.sin(beta * Z) / (beta * h)
    uy = u0 * (1 - E**2) + 0.3 * u0 * (1 - E**2) * np.cos(beta * Z) * np.cos(alpha * Y)
    rng = np.random.default_rng(seed)
    for u in (ux, uy, uz):
        u += amp * u0 * rng.uniform(-1.0, 1.0, u.shape) * (1 - E**2)
    return [np.asfortranarray(u) for u in (ux, uy, uz)]


def developed_state(cfg, spinup: int, device: int, seed: int):
    """Populations of developed particle-free turbulence: FP32 DNS of the
    configuration's channel from the trigger, `spinup` steps.  Returns (f,
    history of [step, peak |<u'w'>|/u*^2, centreline/u*], ms per step)."""
    run = cfg.params("fp32", device=device)
    hist = []
    with pkg.Lattice(run) as lat:
        lat.initpop(*trigger_velocity(cfg.wall, cfg.stream, cfg.span, cfg.h, 18.0 * cfg.ustar, 0.05, seed))
        t0 = time.perf_counter()
        done = 0
        while done < spinup:
            k = min(20000, spinup - done)
            lat.step(k)
            done += k
            st = pkg.statistics(lat.profiles(), cfg.ustar)
            hist.append([done, float(np.abs(st["stress"][:, 1]).max()), float(st["mean"][:, 1].max())])
            print(f"[spinup] step {done}: |u'w'|/u*^2 max {hist[-1][1]:.3f}, centreline/u* {hist[-1][2]:.2f}",
                  flush=True)
        ms = (time.perf_counter() - t0) * 1e3 / max(done, 1)
        return lat.download_f(), hist, ms


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
    ap.add_argument("--start", choices=("poiseuille", "developed"), default="poiseuille")
    ap.add_argument("--spinup", type=int, default=160000, help="FP32 DNS steps before the window (developed)")
    ap.add_argument("--trigger-seed", type=int, default=20240611)
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
    f0 = None
    spin = None
    runs = [(p, p) for p in precs]
    if args.start == "developed":
        f0, hist, ms = developed_state(cfg, args.spinup, args.device, args.trigger_seed)
        spin = dict(steps=args.spinup, fp32_ms_per_step=ms, history=hist)
        runs.insert(1, ("fp64_perturbed", "fp64"))
    res = {}
    for name, p in runs:
        t0 = time.perf_counter()
        fi = f0
        if name == "fp64_perturbed":
            rng = np.random.default_rng(1)
            fi = f0 * (1.0 + 1e-12 * rng.uniform(-1.0, 1.0, f0.shape))
        res[name] = run_one(cfg, p, pos, steps, args.every, args.device, fi)
        print(f"[sweep] {name}: {res[name]['steps_done']} steps, {1e3 * res[name]['s_per_step']:.3f} ms/step, "
              f"fail={res[name]['fail']}, {time.perf_counter() - t0:.0f} s", flush=True)
    lo = steps // 2
    ref = res["fp64"]
    wref = window(ref, lo)
    others = [n for n, _ in runs if n != "fp64"]
    report = dict(
        config=cfg.name, start=args.start, spinup=spin,
        grid_stream_span_wall=[cfg.stream, cfg.span, cfg.wall], spheres=cfg.spheres,
        radius=cfg.radius, visc=cfg.visc, ustar=cfg.ustar, h=cfg.h, steps=steps, every=args.every,
        window=f"samples with step > {lo}", seed=cfg.seed,
        runs={p: dict(ms_per_step=1e3 * r["s_per_step"], steps_done=r["steps_done"], fail=r["fail"], **drift(r))
              for p, r in res.items()},
        fp64=dict(centreline_u_over_ustar=float(wref["mean"].max()) if wref else None,
                  peak_reynolds_stress=float(np.abs(wref["stress"]).max()) if wref else None,
                  mean_drag=wref.get("drag") if wref else None),
        errors={p: compare(res[p], ref, lo) for p in others},
        profiles={p: dict(mean=window(r, lo)["mean"].tolist(), stress=window(r, lo)["stress"].tolist())
                  for p, r in res.items() if window(r, lo)},
        series={p: [dict(step=x["step"], drag=float(x["drag"].mean()), rho_sum=x["rho_sum"],
                         centreline=float(x["mean"].max()), peak_stress=float(np.abs(x["stress"]).max()))
                    for x in r["samples"]] for p, r in res.items()},
    )
    args.out.mkdir(parents=True, exist_ok=True)
    tag = "_developed" if args.start == "developed" else ""
    path = args.out / f"precision_sweep_{cfg.stream}x{cfg.span}x{cfg.wall}{tag}.json"
    path.write_text(json.dumps(report, indent=1))
    print(json.dumps(dict(runs=report["runs"], errors=report["errors"], fp64=report["fp64"]), indent=1))
    print(f"[sweep] report: {path}")


if __name__ == "__main__":
    main()
