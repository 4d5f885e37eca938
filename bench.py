#!/usr/bin/env python
"""Throughput of the D3Q19 channel-flow time step on GB300.

One bench step = one lattice time step (collision + streaming + walls +
periodic wrap) over the whole domain.  Default workload: the large channel
1024 x 512 x 512 (streamwise x spanwise x wall-normal), FP32 arithmetic on
populations stored as FP16 deviations with a fixed scale, nu = 0.0024,
u* = 0.0034, h = 256, seeded Poiseuille + 5 % noise initial state.  The
moving spheres of that configuration are not part of this step yet, so the
workload is named "particle-free".

Printed JSON line (rank 0):
  value      GLUPS over all ranks, device-resident state, CUDA-event timed
  e2e        GLUPS through the C ABI with host buffers: initpop from pinned
             host velocity arrays, the steps (one synchronous lbm_step call
             each, lbm_diag every 250 steps), macrovar back to pinned host
             arrays -- all inside the timed region
  roofline   38 populations x 2 B per node per step over the measured HBM copy
             bandwidth; traffic from the committed ncu capture
  cpu_baseline  the FP64 oracle (C, OpenMP on all host cores) on a slab sample
             of the same channel
  accuracy   FP16-store / FP32 run against FP64 over a 100-step window from
             the same initial state: mean streamwise profile, Reynolds shear
             stress and mass drift
--impl reference  times the CPU implementation (the oracle port; the Fortran
             reference cannot be built on these machines) on the same workload.
"""
from __future__ import annotations

import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))
PKG = "d3q19-single-phase_gb300"
BYTES = {"fp64": 8, "fp32": 4, "fp16": 2}
L2_BYTES = 129 * 2**20


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def committed_traffic(workload: str) -> dict | None:
    """Per-launch DRAM bytes of the step kernels from the committed ncu summary."""
    p = REPO / "profiles" / "dram_traffic.txt"
    if not p.exists():
        return None
    out = {}
    for line in p.read_text().splitlines():
        if "=" in line and not line.lstrip().startswith("#"):
            k, v = (s.strip() for s in line.split("=", 1))
            out[k] = v
    if out.get("workload") != workload:
        return None
    try:
        return {k: float(out[k]) for k in ("even_bytes", "odd_bytes")}
    except (KeyError, ValueError):
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (FileNotFoundError, OSError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "power_w_median": statistics.median(power),
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl"
        try:
            import torch
            if not torch.cuda.is_available():
                backend = "gloo"
            else:
                torch.cuda.set_device(local)
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allmax(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_name(cfg, prec) -> str:
    return f"channel {cfg.stream}x{cfg.span}x{cfg.wall} {prec}-store particle-free ({cfg.name})"


# --------------------------------------------------------------------------
def cpu_sample(orc, cfg, budget_s: float, threads: int, warmup_steps: int = 1, fixed_steps: int | None = None):
    """Time the oracle's OpenMP step on a spanwise slab of the channel.

    Returns (glups, nodes, steps, seconds, shape)."""
    run = cfg.params("fp64")
    p = orc.params_from(run)
    nz = 2
    shape = (cfg.wall, cfg.stream, nz)
    u = orc.channel_velocity(*shape, cfg.uc, cfg.amp, cfg.seed)
    f = orc.initpop(*u)
    orc.run_omp(p, f, warmup_steps, threads)
    t0 = time.perf_counter()
    orc.run_omp(p, f, 1, threads)
    t1 = time.perf_counter() - t0
    nodes = int(np.prod(shape))
    steps = fixed_steps if fixed_steps is not None else max(1, int(budget_s / max(t1, 1e-6)))
    t0 = time.perf_counter()
    orc.run_omp(p, f, steps, threads)
    dt = time.perf_counter() - t0
    return nodes * steps / dt / 1e9, nodes, steps, dt, shape


def run_reference(args, world, rank):
    """--impl reference: the CPU implementation of the step, rank 0 only."""
    if rank != 0:
        return
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle as orc
    pkg = importlib.import_module(PKG)
    cfg = pkg.CHANNEL_CONFIGS[args.config]
    prec = args.precision or cfg.precision
    threads = os.cpu_count() or 1
    run = cfg.params("fp64")
    p = orc.params_from(run)
    # slab sample sized so that warm-up + timed steps take about args.cpu_budget seconds
    shape = (cfg.wall, cfg.stream, 1)
    u = orc.channel_velocity(*shape, cfg.uc, cfg.amp, cfg.seed)
    f = orc.initpop(*u)
    orc.run_omp(p, f, 1, threads)
    t0 = time.perf_counter()
    orc.run_omp(p, f, 2, threads)
    per_plane_step = (time.perf_counter() - t0) / 2
    per_step_budget = args.cpu_budget / max(1, args.steps + args.warmup)
    nz = max(1, min(cfg.span, int(per_step_budget / max(per_plane_step, 1e-9))))
    shape = (cfg.wall, cfg.stream, nz)
    u = orc.channel_velocity(*shape, cfg.uc, cfg.amp, cfg.seed)
    f = orc.initpop(*u)
    orc.run_omp(p, f, args.warmup, threads)
    t0 = time.perf_counter()
    orc.run_omp(p, f, args.steps, threads)
    dt = time.perf_counter() - t0
    nodes = int(np.prod(shape))
    glups = nodes * args.steps / dt / 1e9
    sample = (f"each step = one FP64 time step of the oracle port (no Fortran compiler on these machines) "
              f"on a {cfg.stream}x{nz}x{cfg.wall} slab ({nodes} nodes) of the {cfg.stream}x{cfg.span}x{cfg.wall} "
              f"channel, two-lattice push, {threads} OpenMP threads")
    line = {
        "impl": "reference", "metric": "GLUPS (lattice updates per second / 1e9)", "value": round(glups, 6),
        "unit": "GLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(cfg, prec), "sample_nodes": nodes},
        "cpu_baseline": {"value": round(glups, 6), "unit": "GLUPS", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(glups, 6), "unit": "GLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
def run_gpu(args, world, rank, local):
    import torch

    pkg = importlib.import_module(PKG)
    cfg = pkg.CHANNEL_CONFIGS[args.config]
    prec = args.precision or cfg.precision
    N = cfg.nodes
    bpn = 38 * BYTES[prec]
    run = cfg.params(prec, device=local, flags=pkg.FLAG_SIMPLE_STEP if args.simple else 0)
    torch.cuda.set_device(local)
    lat = pkg.Lattice(run)
    lat.init_channel(cfg.uc, cfg.amp, cfg.seed)
    log(f"[bench] rank {rank}: {workload_name(cfg, prec)}, {N} nodes, {lat.device_bytes() / 1e9:.2f} GB on device")
    lat.step(args.warmup)
    stream = torch.cuda.ExternalStream(lat.stream())
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    parity0 = lat.step_count() % 2
    for k in range(args.steps):
        evs[k].record(stream)
        lat.step_async(1)
    evs[-1].record(stream)
    lat.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop()
    per = np.array([evs[k].elapsed_time(evs[k + 1]) for k in range(args.steps)])   # ms
    total_ms = float(evs[0].elapsed_time(evs[-1]))
    total_ms = allmax(world, total_ms)
    value = world * N * args.steps / (total_ms / 1e3) / 1e9
    st = lat.diag()
    if st.nonfinite:
        raise RuntimeError("non-finite populations after the timed steps")

    # roofline of the step kernels (even/odd AA launches alternate)
    peaks = measured_peaks()
    even = per[(np.arange(args.steps) + parity0) % 2 == 0]
    odd = per[(np.arange(args.steps) + parity0) % 2 == 1]
    alg = bpn * N
    achieved = alg / (per.mean() / 1e3) / 1e9
    traffic = committed_traffic(workload_name(cfg, prec))
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / peaks["hbm_gbs"], 4),
            "traffic": (round((traffic["even_bytes"] + traffic["odd_bytes"]) / 2) if traffic else None),
            "peak_source": f"{peaks['source']} (MEASURED_PEAKS.json hbm_gbs)",
            "algorithmic_bytes_per_launch": alg,
            "kernels": {"even_local": {"ms": round(float(even.mean()), 4),
                                       "achieved": round(alg / (even.mean() / 1e3) / 1e9, 1)},
                        "odd_neighbour": {"ms": round(float(odd.mean()), 4),
                                          "achieved": round(alg / (odd.mean() / 1e3) / 1e9, 1)}}}

    accuracy = None
    if rank == 0 and args.accuracy_steps > 0 and prec != "fp64":
        accuracy = accuracy_window(pkg, cfg, prec, args.accuracy_steps, local, lat)
    lat.close()

    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(pkg, torch, cfg, prec, args.steps, local, world)

    cpu = None
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, str(REPO / "oracle"))
        import oracle as orc
        threads = os.cpu_count() or 1
        g, nodes, steps, dt, shape = cpu_sample(orc, cfg, args.cpu_budget, threads)
        cpu = {"value": round(g, 6), "unit": "GLUPS", "cores": threads, "kind": "port",
               "sample": f"FP64 oracle port (OpenMP two-lattice push) on a {shape[1]}x{shape[2]}x{shape[0]} slab "
                         f"of the same channel, {steps} steps in {dt:.1f} s"}

    if rank == 0:
        line = {
            "metric": "GLUPS (lattice updates per second / 1e9); FP16-store/FP32 vs FP64 error in `accuracy`",
            "value": round(value, 4), "unit": "GLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec != "fp64" else "f64",
            "data": "synthetic (seeded Poiseuille + uniform noise initial state)",
            "config": {"workload": workload_name(cfg, prec), "storage": prec, "nodes": N,
                       "grid_stream_span_wall": [cfg.stream, cfg.span, cfg.wall], "visc": cfg.visc,
                       "ustar": cfg.ustar, "h": cfg.h, "mrt": "MRTtype 1 (para.f90)",
                       "l2": f"populations {N * 19 * BYTES[prec] / 1e9:.1f} GB >> 129 MB L2, no flush needed",
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
            "roofline": roof, "clocks": clocks, "gpu_launches": args.steps,
            "e2e": e2e, "cpu_baseline": cpu, "accuracy": accuracy,
        }
        print(json.dumps(line), flush=True)


def accuracy_window(pkg, cfg, prec, steps, device, lat_lp):
    """FP64 vs the low-precision run over `steps` steps from the same initial
    state (the FP64 spot check of the large configuration)."""
    out = {}
    res = {}
    for p in ("fp64", prec):
        with pkg.Lattice(cfg.params(p, device=device)) as lat:
            lat.init_channel(cfg.uc, cfg.amp, cfg.seed)
            d0 = lat.diag()
            lat.step(steps)
            d1 = lat.diag()
            res[p] = (pkg.statistics(lat.profiles(), cfg.ustar), d1.rho_sum - d0.rho_sum)
    ref, lp = res["fp64"][0], res[prec][0]
    mref = ref["mean"][:, 1]
    out["steps"] = steps
    out["mean_profile_rel_err"] = float(np.abs(lp["mean"][:, 1] - mref).max() / np.abs(mref).max())
    sref = ref["stress"][:, 1]
    out["reynolds_stress_rel_err"] = float(np.abs(lp["stress"][:, 1] - sref).max() / max(np.abs(sref).max(), 1e-30))
    out["reynolds_stress_max_fp64"] = float(np.abs(sref).max())
    out["mass_drift_fp64"] = res["fp64"][1]
    out[f"mass_drift_{prec}"] = res[prec][1]
    return out


def e2e_run(pkg, torch, cfg, prec, steps, device, world):
    """GLUPS through the public C ABI with pinned host buffers in and out."""
    N = cfg.nodes
    shape = (cfg.wall, cfg.stream, cfg.span)
    host = [torch.empty(N, dtype=torch.float64, pin_memory=True) for _ in range(4)]
    arrs = [h.numpy().reshape(shape, order="F") for h in host]
    lib = pkg.load_library()
    rc = lib.lbm_channel_velocity(cfg.wall, cfg.stream, cfg.span, cfg.uc, cfg.amp, cfg.seed,
                                  *(pkg._dptr(a) for a in arrs[:3]))
    if rc != 0:
        raise RuntimeError("lbm_channel_velocity failed")
    lat = pkg.Lattice(cfg.params(prec, device=device))
    ndiag = 250
    diag_bytes = (cfg.wall * 64 * pkg.PROFILE_COLS + 1024 * 5) * 8
    barrier(world)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lat.initpop(arrs[0], arrs[1], arrs[2])
    ndiags = 0
    for k in range(1, steps + 1):
        lat.step(1)
        if k % ndiag == 0:
            lat.diag()
            ndiags += 1
    lib.lbm_macrovar(lat._ctx, *(pkg._dptr(a) for a in arrs))
    dt = time.perf_counter() - t0
    dt = allmax(world, dt)
    lat.close()
    return {"value": round(world * N * steps / dt / 1e9, 4), "unit": "GLUPS",
            "h2d_bytes_per_step": int(3 * N * 8 / steps),
            "d2h_bytes_per_step": int((4 * N * 8 + ndiags * diag_bytes) / steps),
            "path": "lbm_initpop(host u) -> lbm_step(1) x steps (+lbm_diag every 250) -> lbm_macrovar(host)",
            "seconds": round(dt, 3)}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=1000)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--config", default="c4")
    ap.add_argument("--precision", choices=tuple(BYTES), default=None)
    ap.add_argument("--accuracy-steps", type=int, default=100)
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU work for the CPU baseline")
    ap.add_argument("--grid", type=int, nargs=3, metavar=("STREAM", "SPAN", "WALL"), default=None,
                    help="override the lattice (streamwise spanwise wall-normal), e.g. for a small ncu capture")
    ap.add_argument("--simple", action="store_true", help="one-node-per-thread step kernels (A/B reference)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    world, rank, local = dist_setup()
    if args.grid:
        import dataclasses
        pkg = importlib.import_module(PKG)
        c = pkg.CHANNEL_CONFIGS[args.config]
        pkg.CHANNEL_CONFIGS[args.config] = dataclasses.replace(
            c, stream=args.grid[0], span=args.grid[1], wall=args.grid[2], h=args.grid[2] / 2,
            name=f"{c.name}@{args.grid[0]}x{args.grid[1]}x{args.grid[2]}")
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
