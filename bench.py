#!/usr/bin/env python
"""Throughput of the D3Q19 channel-flow time step on GB300.

One bench step = one lattice time step (collision + streaming + walls +
periodic wrap, and with spheres the interpolated bounce-back, momentum
exchange, Newton-Euler update and refilling) over the whole domain.  Default
workload: the large particle-laden channel 1024 x 512 x 512 (streamwise x
spanwise x wall-normal) with 16384 spheres of radius 8 (density ratio 2,
seeded placement with >= 2-node gaps and >= 1 node from the walls), FP32
arithmetic on populations stored as FP16 deviations with a fixed scale,
nu = 0.0024, u* = 0.0034, h = 256, seeded Poiseuille + 5 % noise initial
state.  --no-particles leaves the spheres out.

Printed JSON line (rank 0):
  value      GLUPS over all ranks: fluid-node updates per second / 1e9 (the
             nodes inside spheres are not counted, as the reference skips
             them in its collision, collision.f90:54), device-resident state,
             CUDA-event timed; `all_nodes_glups` counts every lattice node
  e2e        fluid-node GLUPS through the C ABI with pinned host buffers, one
             job per pass: initpop from host velocity arrays (+ the spheres'
             state), then per step one synchronous lbm_step call (it reads
             back the step's status) and the step's result -- the spheres'
             positions, velocities, forces and torques -- to the host,
             lbm_diag every 250 steps, the plane statistics at the end; the
             median of three timed passes after one untimed pass;
             `fields_out` times the full-field download (macrovar) apart
  roofline   38 populations x 2 B per fluid node per step over the measured
             HBM copy bandwidth, for the step kernel and for the whole step;
             traffic from the committed ncu capture
  cpu_baseline  the FP64 oracle (C, OpenMP on all host cores) on a bounded
             sample of the same channel (with spheres: a 64^3 box at the
             channel's sphere volume fraction)
  gpu_launches  kernels the library launched in the timed steps, counted by
             the library itself (lbm_step_launches)
  accuracy   FP16-store / FP32 run against FP64 over a 100-step window from
             the same initial state: mean streamwise profile, Reynolds shear
             stress, mass drift and the spheres' forces and velocities
--impl reference  times the CPU implementation (the oracle port; the Fortran
             reference cannot be built on these machines) on the same workload,
             with the same metric; that arm loads only the oracle library.
"""
from __future__ import annotations

import argparse
import ctypes
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
METRIC = "GLUPS (fluid-node lattice updates per second / 1e9)"
BYTES = {"fp64": 8, "fp32": 4, "fp16": 2}
L2_BYTES = 129 * 2**20
# FP64 instructions per node of the FP64 step kernels (DADD + DFMA + DMUL),
# counted by ncu on one odd-step launch
FP64_INST_PER_NODE = 215
FP64_PROFILE = "profiles/step_fp64_k_step_odd_256x128x128.md"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def peak_gbs_glups(hbm_gbs: float, bytes_per_node: int) -> float:
    return hbm_gbs * 1e9 / bytes_per_node / 1e9


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
        res = {k: float(out[k]) for k in ("even_bytes", "odd_bytes")}
    except (KeyError, ValueError):
        return None
    if "measured_on" in out:
        res["basis"] = (f"ncu dram__bytes of {out['measured_on']}, x {out.get('scale', '?')} "
                        "(profiles/dram_traffic.txt)")
    return res


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


def workload_name(cfg, prec, spheres=True) -> str:
    if cfg.spheres and spheres:
        return (f"channel {cfg.stream}x{cfg.span}x{cfg.wall} {prec}-store, {cfg.spheres} spheres r={cfg.radius:g} "
                f"({cfg.name})")
    return f"channel {cfg.stream}x{cfg.span}x{cfg.wall} {prec}-store particle-free ({cfg.name})"


def sphere_positions(pkg, cfg):
    """Seeded placement of the configuration's spheres: >= 2-node gaps, >= 1 node from the walls."""
    return pkg.place_spheres(cfg.wall, cfg.stream, cfg.span, cfg.spheres, cfg.radius, gap=2.0, wall_gap=1.0,
                             seed=cfg.seed)


# --------------------------------------------------------------------------
def cpu_sample(orc, cfg, budget_s: float, threads: int, spheres: bool):
    """Time the oracle on a bounded sample of the workload.

    Particle-free: a 2-plane spanwise slab of the channel, OpenMP push.
    With spheres: a 64^3 box at the channel's sphere volume fraction, placed
    by the oracle's own seeded placement (fluid push on OpenMP threads,
    sphere steps serial).  Only fluid nodes count as updates.  Returns
    (glups, fluid nodes, steps, seconds, description)."""
    run = cfg.params("fp64")
    p = orc.params_from(run)
    if spheres and cfg.spheres:
        shape = (64, 64, 64)
        n = max(1, round(cfg.spheres * 64**3 / cfg.nodes))
        pos = orc.place_spheres(*shape, n, cfg.radius, gap=2.0, wall_gap=1.0, seed=cfg.seed)
        u = orc.channel_velocity(*shape, cfg.uc, cfg.amp, cfg.seed)
        f = orc.initpop(*u)
        sp = orc.Spheres(pos, radius=cfg.radius, rho_ratio=2.0)
        f, owner, _, _ = orc.particle_run(p, sp, f, 1)
        t0 = time.perf_counter()
        f, owner, _, _ = orc.particle_run(p, sp, f, 1, owner=owner)
        t1 = time.perf_counter() - t0
        steps = max(1, int(budget_s / max(t1, 1e-6)))
        fluid0 = int((owner == -1).sum())
        t0 = time.perf_counter()
        _, owner, _, _ = orc.particle_run(p, sp, f, steps, owner=owner)
        dt = time.perf_counter() - t0
        nodes = 0.5 * (fluid0 + int((owner == -1).sum()))
        desc = (f"FP64 oracle port, 64x64x64 box with {n} spheres r={cfg.radius:g} (the channel's volume fraction; "
                f"{nodes:.0f} fluid nodes), {steps} steps in {dt:.1f} s")
        return nodes * steps / dt / 1e9, nodes, steps, dt, desc
    shape = (cfg.wall, cfg.stream, 2)
    u = orc.channel_velocity(*shape, cfg.uc, cfg.amp, cfg.seed)
    f = orc.initpop(*u)
    orc.run_omp(p, f, 1, threads)
    t0 = time.perf_counter()
    orc.run_omp(p, f, 1, threads)
    t1 = time.perf_counter() - t0
    nodes = int(np.prod(shape))
    steps = max(1, int(budget_s / max(t1, 1e-6)))
    t0 = time.perf_counter()
    orc.run_omp(p, f, steps, threads)
    dt = time.perf_counter() - t0
    desc = (f"FP64 oracle port (OpenMP two-lattice push) on a {shape[1]}x{shape[2]}x{shape[0]} slab of the same "
            f"channel, {steps} steps in {dt:.1f} s")
    return nodes * steps / dt / 1e9, nodes, steps, dt, desc


def run_reference(args, world, rank):
    """--impl reference: the CPU implementation of the step, rank 0 only.

    The Fortran reference cannot be built on these machines (no Fortran
    compiler, no MPI), so the CPU implementation timed is the FP64 oracle port
    with all host threads; each step is one time step of a bounded sample of
    the workload, sized so that warm-up + timed steps take ~cpu_budget s."""
    if rank != 0:
        return
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle as orc
    pkg = importlib.import_module(PKG)      # configuration table only; the library is not loaded
    cfg = pkg.CHANNEL_CONFIGS[args.config]
    prec = args.precision or cfg.precision
    threads = os.cpu_count() or 1
    spheres = bool(cfg.spheres) and not args.no_particles
    per_step = args.cpu_budget / max(1, args.steps + args.warmup)
    g, nodes, steps, dt, desc = cpu_sample(orc, cfg, per_step * (args.steps + args.warmup), threads, spheres)
    sample = f"each step = one time step of: {desc}; {threads} host threads"
    line = {
        "impl": "reference", "metric": METRIC, "value": round(g, 6),
        "unit": "GLUPS", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / max(steps, 1) * 1e3, 4), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_name(cfg, prec, spheres), "sample_fluid_nodes": nodes, "sample_steps": steps},
        "cpu_baseline": {"value": round(g, 6), "unit": "GLUPS", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": round(g, 6), "unit": "GLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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
    spheres = bool(cfg.spheres) and not args.no_particles
    wname = workload_name(cfg, prec, spheres)
    torch.cuda.set_device(local)
    lat = pkg.Lattice(run)
    lat.init_channel(cfg.uc, cfg.amp, cfg.seed)
    pos = None
    pflags = pkg.PFLAG_Q_FP64 if args.qfp64 else 0
    if spheres:
        pos = sphere_positions(pkg, cfg)
        lat.set_particles(pos, cfg.radius, 2.0, flags=pflags)
    log(f"[bench] rank {rank}: {wname}, {N} nodes, {lat.device_bytes() / 1e9:.2f} GB on device")
    lat.step(args.warmup)
    fluid0 = lat.diag().nfluid
    stream = torch.cuda.ExternalStream(lat.stream())
    evs = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    sampler = ClockSampler(local)
    barrier(world)
    torch.cuda.synchronize()
    sampler.start()
    time.sleep(0.3)
    launches0 = lat.step_launches()
    lat.timing_enable(args.steps)
    for k in range(args.steps):
        evs[k].record(stream)
        lat.step_async(1)
    evs[-1].record(stream)
    launches = lat.step_launches() - launches0
    lat.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop()
    total_ms = float(evs[0].elapsed_time(evs[-1]))
    total_ms = allmax(world, total_ms)
    st = lat.diag()
    if st.nonfinite:
        raise RuntimeError("non-finite populations after the timed steps")
    # fluid nodes: the mean of the counts before and after the timed steps
    # (sphere surfaces cover and uncover a few nodes per step)
    NF = 0.5 * (fluid0 + st.nfluid)
    value = world * NF * args.steps / (total_ms / 1e3) / 1e9
    value_all = world * N * args.steps / (total_ms / 1e3) / 1e9

    # roofline of the fluid step kernel (even/odd AA launches alternate), timed
    # by events the library records around each launch inside the timed loop;
    # algorithmic bytes = 38 populations per fluid node
    tm = lat.timing()
    peaks = measured_peaks()
    ev_ms = tm["even_ms"] / max(tm["even"], 1)
    od_ms = tm["odd_ms"] / max(tm["odd"], 1)
    fluid_ms = (tm["even_ms"] + tm["odd_ms"]) / max(tm["even"] + tm["odd"], 1)
    alg = bpn * NF
    achieved = alg / (fluid_ms / 1e3) / 1e9
    step_ach = alg / (total_ms / args.steps / 1e3) / 1e9
    traffic = committed_traffic(wname)
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / peaks["hbm_gbs"], 4),
            "traffic": (round((traffic["even_bytes"] + traffic["odd_bytes"]) / 2) if traffic else None),
            "traffic_basis": traffic.get("basis") if traffic else None,
            "peak_source": f"{peaks['source']} (MEASURED_PEAKS.json hbm_gbs)",
            "kernel": ("k_step_rows" if prec != "fp64" and not args.simple else "k_step_even/odd")
                      + " (even/odd AA launches alternate)",
            "algorithmic_bytes_per_launch": round(alg),
            "algorithmic_basis": f"38 populations x {BYTES[prec]} B per fluid node ({NF:.0f} fluid nodes)",
            "whole_step": {"achieved": round(step_ach, 1), "frac": round(step_ach / peaks["hbm_gbs"], 4),
                           "ms": round(total_ms / args.steps, 4)},
            "all_nodes": {"nodes": N, "algorithmic_bytes_per_launch": bpn * N,
                          "achieved": round(bpn * N / (fluid_ms / 1e3) / 1e9, 1),
                          "frac": round(bpn * N / (fluid_ms / 1e3) / 1e9 / peaks["hbm_gbs"], 4)},
            "kernels": {"even_local": {"ms": round(ev_ms, 4), "achieved": round(alg / (ev_ms / 1e3) / 1e9, 1)},
                        "odd_neighbour": {"ms": round(od_ms, 4), "achieved": round(alg / (od_ms / 1e3) / 1e9, 1)},
                        "spheres_per_step_ms": round(tm["particle_ms"] / max(tm["even"] + tm["odd"], 1), 4)}}
    if spheres:
        ns, nl, nr = lat.particle_counts()
        roof["spheres"] = {"solid_nodes": ns, "links_last_step": nl, "refills_last_step": nr}
    if prec == "fp64":
        # the FP64 step is bound by the FP64 pipe (2 instructions per SM per
        # cycle on GB300), not by bytes: the min(byte, FP64) roofline
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        mhz = clocks.get("sm_mhz") or 2070.0
        peak_inst = 2.0 * sms * mhz * 1e6
        per_node = FP64_INST_PER_NODE
        ach_inst = per_node * N / (fluid_ms / 1e3)
        roof["fp64_pipe"] = {"instructions_per_node": per_node, "source": FP64_PROFILE,
                             "peak_ginst_s": round(peak_inst / 1e9, 1), "achieved_ginst_s": round(ach_inst / 1e9, 1),
                             "frac": round(ach_inst / peak_inst, 4),
                             "glups_roof_fp64": round(peak_inst / per_node / 1e9, 3),
                             "glups_roof_bytes": round(peak_gbs_glups(peaks["hbm_gbs"], bpn), 3),
                             "binding": "fp64 pipe"}

    lat.close()
    accuracy = None
    if rank == 0 and args.accuracy_steps > 0 and prec != "fp64":
        accuracy = accuracy_window(pkg, cfg, prec, args.accuracy_steps, local, pos, pflags)

    e2e = None
    if not args.no_e2e:
        e2e = e2e_run(pkg, torch, cfg, prec, args.steps, local, world, pos, pflags)

    cpu = None
    if rank == 0 and not args.no_cpu:
        sys.path.insert(0, str(REPO / "oracle"))
        import oracle as orc
        threads = os.cpu_count() or 1
        g, nodes, steps, dt, desc = cpu_sample(orc, cfg, args.cpu_budget, threads, spheres)
        cpu = {"value": round(g, 6), "unit": "GLUPS", "cores": threads, "kind": "port", "sample": desc}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 4), "unit": "GLUPS", "all_nodes_glups": round(value_all, 4), "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32" if prec != "fp64" else "f64",
            "data": "synthetic (seeded Poiseuille + uniform noise initial state)",
            "config": {"workload": wname, "storage": prec, "nodes": N, "fluid_nodes": round(NF),
                       "grid_stream_span_wall": [cfg.stream, cfg.span, cfg.wall], "visc": cfg.visc,
                       "ustar": cfg.ustar, "h": cfg.h, "mrt": "MRTtype 1 (para.f90)" + (f", s16={cfg.s16}" if cfg.s16 else ""),
                       "link_fractions": "fp64" if (args.qfp64 or prec == "fp64") else "fp32",
                       "l2": f"populations {N * 19 * BYTES[prec] / 1e9:.1f} GB >> 129 MB L2, no flush needed",
                       "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
            "roofline": roof, "clocks": clocks, "gpu_launches": launches,
            "e2e": e2e, "cpu_baseline": cpu, "accuracy": accuracy,
        }
        print(json.dumps(line), flush=True)


def accuracy_window(pkg, cfg, prec, steps, device, pos, pflags=0):
    """FP64 vs the low-precision run over `steps` steps from the same initial
    state (the FP64 spot check of the large configuration)."""
    out = {}
    res = {}
    for p in ("fp64", prec):
        with pkg.Lattice(cfg.params(p, device=device)) as lat:
            lat.init_channel(cfg.uc, cfg.amp, cfg.seed)
            if pos is not None:
                lat.set_particles(pos, cfg.radius, 2.0, flags=pflags)
            d0 = lat.diag()
            lat.step(steps)
            d1 = lat.diag()
            part = lat.particles() if pos is not None else None
            res[p] = (pkg.statistics(lat.profiles(), cfg.ustar), d1.rho_sum - d0.rho_sum, part,
                      d1.rho_sum / max(d1.nfluid, 1) - d0.rho_sum / max(d0.nfluid, 1))
    ref, lp = res["fp64"][0], res[prec][0]
    mref = ref["mean"][:, 1]
    out["steps"] = steps
    out["mean_profile_rel_err"] = float(np.abs(lp["mean"][:, 1] - mref).max() / np.abs(mref).max())
    sref = ref["stress"][:, 1]
    out["reynolds_stress_rel_err"] = float(np.abs(lp["stress"][:, 1] - sref).max() / max(np.abs(sref).max(), 1e-30))
    out["reynolds_stress_max_fp64"] = float(np.abs(sref).max())
    out["mass_drift_fp64"] = res["fp64"][1]
    out[f"mass_drift_{prec}"] = res[prec][1]
    # with spheres the fluid node set changes as surfaces cover and uncover
    # nodes; the mean density over the fluid nodes is the comparable figure
    out["mean_density_drift_fp64"] = res["fp64"][3]
    out[f"mean_density_drift_{prec}"] = res[prec][3]
    if pos is not None:
        a, b = res[prec][2], res["fp64"][2]
        fb = b["force"]
        out["particle_force_rel_err"] = float(np.abs(a["force"] - fb).max() / max(np.abs(fb).max(), 1e-300))
        out["particle_force_mean_rel_err"] = float(np.abs(a["force"].mean(0) - fb.mean(0)).max()
                                                   / max(np.abs(fb.mean(0)).max(), 1e-300))
        out["particle_velocity_rel_err"] = float(np.abs(a["vel"] - b["vel"]).max() / max(np.abs(b["vel"]).max(), 1e-300))
    return out


def e2e_run(pkg, torch, cfg, prec, steps, device, world, pos=None, pflags=0, passes=3):
    """GLUPS through the public C ABI with pinned host buffers.  A pass is one
    job: the initial velocity field goes in from pinned host arrays
    (lbm_initpop), the spheres' state with it (lbm_particles_set); every step
    is one synchronous lbm_step call, which reads back the step's status
    flags, followed by the step's result -- the spheres' positions,
    velocities, forces and torques -- into pinned host arrays
    (lbm_particles_get); lbm_diag every 250 steps; the run's plane statistics
    (lbm_profiles) at the end.  The download of the full macroscopic fields
    (lbm_macrovar, 4 FP64 arrays) is timed after each pass and reported
    beside the value (`fields_out`), not inside it."""
    N = cfg.nodes
    shape = (cfg.wall, cfg.stream, cfg.span)
    host = [torch.empty(N, dtype=torch.float64, pin_memory=True) for _ in range(4)]
    arrs = [h.numpy().reshape(shape, order="F") for h in host]
    npart = 0 if pos is None else len(pos)
    pres = [torch.empty((max(npart, 1), 3), dtype=torch.float64, pin_memory=True).numpy() for _ in range(5)]
    lib = pkg.load_library()

    def velocity():
        if lib.lbm_channel_velocity(cfg.wall, cfg.stream, cfg.span, cfg.uc, cfg.amp, cfg.seed,
                                    *(pkg._dptr(a) for a in arrs[:3])) != 0:
            raise RuntimeError("lbm_channel_velocity failed")

    def step_result():
        if npart and lib.lbm_particles_get(lat._ctx, *(pkg._dptr(a) for a in pres)) != 0:
            raise RuntimeError("lbm_particles_get failed")

    velocity()
    lat = pkg.Lattice(cfg.params(prec, device=device))
    ndiag = 250
    # untimed warm-up of the same calls: the first device access to each host
    # page of the buffers costs far more than later ones on this platform
    lat.initpop(arrs[0], arrs[1], arrs[2])
    if npart:
        lat.set_particles(pos, cfg.radius, 2.0, flags=pflags)
    lat.step(1)
    step_result()
    lat.profiles()
    lib.lbm_macrovar(lat._ctx, *(pkg._dptr(a) for a in arrs))
    times, fields = [], []
    ndiags = 0
    for _ in range(passes):
        velocity()                               # macrovar wrote over the velocity inputs
        barrier(world)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        lat.initpop(arrs[0], arrs[1], arrs[2])
        if npart:
            lat.set_particles(pos, cfg.radius, 2.0, flags=pflags)
        ndiags = 0
        for k in range(1, steps + 1):
            lat.step(1)
            step_result()
            if k % ndiag == 0:
                lat.diag()
                ndiags += 1
        lat.profiles()
        times.append(allmax(world, time.perf_counter() - t0))
        t1 = time.perf_counter()
        lib.lbm_macrovar(lat._ctx, *(pkg._dptr(a) for a in arrs))
        fields.append(allmax(world, time.perf_counter() - t1))
    dt = statistics.median(times)
    df = statistics.median(fields)
    nf = lat.diag().nfluid                       # fluid nodes (after the run)
    lat.close()
    status_bytes = 8                             # the error flags lbm_step reads back
    prof_bytes = cfg.wall * pkg.PROFILE_COLS * 8
    diag_bytes = ctypes.sizeof(pkg.LBMStats)
    return {"value": round(world * nf * steps / dt / 1e9, 4), "unit": "GLUPS",
            "h2d_bytes_per_step": int((3 * N * 8 + npart * 3 * 8) / steps),
            "d2h_bytes_per_step": int(status_bytes + 5 * npart * 3 * 8 + (ndiags * diag_bytes + prof_bytes) / steps),
            "path": ("lbm_initpop(host u)" + (" + lbm_particles_set(host)" if npart else "")
                     + " -> [lbm_step(1)" + (" + lbm_particles_get(host)" if npart else "")
                     + "] x steps (+lbm_diag every 250) -> lbm_profiles(host)"),
            "seconds": round(dt, 3), "pass_seconds": [round(t, 3) for t in times],
            "fields_out": {"call": "lbm_macrovar(host rho, ux, uy, uz)", "bytes": 4 * N * 8,
                           "seconds": round(df, 3),
                           "value_with_fields_out": round(world * nf * steps / (dt + df) / 1e9, 4)},
            "timing": f"median of {passes} timed passes after one untimed pass of the same calls"}


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=1000)
    ap.add_argument("--impl", choices=("gb300", "reference"), default="gb300")
    ap.add_argument("--config", default="spheres-1024x512x512")
    ap.add_argument("--precision", choices=tuple(BYTES), default=None)
    ap.add_argument("--accuracy-steps", type=int, default=100)
    ap.add_argument("--cpu-budget", type=float, default=15.0, help="seconds of CPU work for the CPU baseline")
    ap.add_argument("--grid", type=int, nargs=3, metavar=("STREAM", "SPAN", "WALL"), default=None,
                    help="override the lattice (streamwise spanwise wall-normal), e.g. for a small ncu capture")
    ap.add_argument("--simple", action="store_true", help="one-node-per-thread step kernels (A/B reference)")
    ap.add_argument("--no-particles", action="store_true", help="leave the configuration's spheres out")
    ap.add_argument("--qfp64", action="store_true",
                    help="boundary-link fractions q in FP64 for FP32/FP16 storage (default FP32)")
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
        nodes = args.grid[0] * args.grid[1] * args.grid[2]
        pkg.CHANNEL_CONFIGS[args.config] = dataclasses.replace(
            c, stream=args.grid[0], span=args.grid[1], wall=args.grid[2], h=args.grid[2] / 2,
            spheres=round(c.spheres * nodes / c.nodes),      # same sphere volume fraction
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
