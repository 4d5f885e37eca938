"""The C++ driver (the reference's main.f90 loop on the C ABI) on the GPU.

Particle checkpoints are the reference's endrunpart2D files
(savecntdpart / loadcntdpart, saveload.f90:604-693).

Checks: a sphere run through the driver equals the same calls made through
the Python binding (same checkpoint header; populations and sphere state equal
to rounding: the bounce-back kernel lists a sphere's candidate rows with a
shared-memory counter, so which lane sums which links -- and the rounding of
the per-sphere force sums -- varies from run to run, and two identical runs
agree to the last bits only, relative L-inf <= 1e-12 / 1e-10); a run stopped
and continued from its endrunflow/endrunpart checkpoints equals the
uninterrupted run across an odd restart step and the every-100-steps mean
density removal (relative L-inf <= 1e-11 in the populations, 1e-10 in the
sphere state, FP64 storage: the checkpoint holds f = w + (f - w), whose
round trip is exact to one rounding of w); diag.dat and profiles2.dat have the
reference's row layout.
"""
from __future__ import annotations

import struct
import subprocess
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPE = (24, 32, 22)                 # reference axes: wall normal, streamwise, spanwise
COMMON = dict(visc=0.02, ustar=0.005, h=12.0, uc=0.04, amp=0.05, seed=11, npart=3, rad=4.0, rhopart=2.0,
              iseedp=7, precision="fp64")


def records(path: Path) -> list[bytes]:
    """Fortran sequential unformatted records (4-byte markers)."""
    data = path.read_bytes()
    out, k = [], 0
    while k < len(data):
        (n,) = struct.unpack_from("<i", data, k)
        out.append(data[k + 4:k + 4 + n])
        assert struct.unpack_from("<i", data, k + 4 + n)[0] == n
        k += 8 + n
    return out


def part_state(path: Path, npart: int) -> dict:
    """endrunpart2D (savecntdpart, saveload.f90:604-647) for one process."""
    r = records(path)
    assert len(r) == 6
    head = np.frombuffer(r[0], dtype="<i4")
    msize = len(head) - 1
    assert head[0] == npart and msize == 10 * npart
    ids = head[1:npart + 1] - 1
    assert sorted(ids) == list(range(npart)) and not head[npart + 1:].any()
    nodes = np.frombuffer(r[1], dtype="<i4")
    ib, isn = nodes[:len(nodes) // 2], nodes[len(nodes) // 2:]

    def local(rec):
        a = np.frombuffer(rec, dtype="<f8").reshape(2, msize, 3)
        assert not a[:, npart:].any()
        out = np.empty((2, npart, 3))
        out[:, ids] = a[:, :npart]
        return out

    yp_th, fp_tp, acc = local(r[2]), local(r[3]), local(r[4])
    g = np.frombuffer(r[5], dtype="<f8").reshape(3, npart, 3)
    assert np.array_equal(yp_th[0], g[0]) and not yp_th[1].any()
    return {"pos": g[0], "vel": g[1], "omg": g[2], "fprev": fp_tp[0], "tprev": fp_tp[1],
            "dwdt": acc[0], "domgdt": acc[1], "ibnodes": ib, "isnodes": isn}


def flow(path: Path) -> np.ndarray:
    r = records(path)
    return np.frombuffer(b"".join(r[1:]), dtype="<f8")


def run_driver(exe: Path, out: Path, **kw) -> str:
    out.mkdir(parents=True, exist_ok=True)
    args = [str(exe), f"nx={SHAPE[0]}", f"ny={SHAPE[1]}", f"nz={SHAPE[2]}", f"out={out}"]
    args += [f"{k}={v}" for k, v in kw.items()]
    res = subprocess.run(args, capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    return res.stdout


@pytest.fixture(scope="module")
def driver():
    import importlib
    b = importlib.import_module("d3q19-single-phase_gb300._build")
    return b.build_driver()


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def check_node_flags(ps: dict, nsolid: int) -> None:
    """ibnodes 1 solid / -1 fluid, isnodes the owning sphere: the nodes whose
    centre lies clearly inside sphere k (reference layout, node ix at ix - 1/2)."""
    nx, ny, nz = SHAPE
    ib = ps["ibnodes"].reshape(nz, ny, nx)             # Fortran (lx, ly, lz) read C-order
    isn = ps["isnodes"].reshape(nz, ny, nx)
    assert set(np.unique(ib)) <= {-1, 1} and int((ib == 1).sum()) == nsolid
    assert np.array_equal(ib == 1, isn > 0)
    iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    for k, c in enumerate(ps["pos"]):
        d = [ix + 0.5 - c[0], iy + 0.5 - c[1], iz + 0.5 - c[2]]
        d[1] = (d[1] + ny / 2) % ny - ny / 2
        d[2] = (d[2] + nz / 2) % nz - nz / 2
        r2 = d[0] ** 2 + d[1] ** 2 + d[2] ** 2
        assert (isn[r2 < 4.0 ** 2 - 0.1] == k + 1).all()
        assert not (isn[r2 > 4.0 ** 2 + 0.1] == k + 1).any()


def test_part_checkpoint_round_trip(pkg, tmp_path):
    """lbm_save_part -> lbm_load_part in a fresh context: state, history and
    node flags come back, and the next steps equal those of the original."""
    nx, ny, nz = SHAPE
    force = COMMON["ustar"] ** 2 / COMMON["h"]
    run = pkg.RunParams(nx=nx, ny=ny, nz=nz, visc=COMMON["visc"], force_y=force, mrt_type=1,
                        precision=pkg.PRECISIONS["fp64"])
    pos = pkg.place_spheres(nx, ny, nz, 3, 4.0, gap=2.0, wall_gap=1.0, seed=7)
    with pkg.Lattice(run) as lat:
        lat.init_channel(COMMON["uc"], COMMON["amp"], COMMON["seed"])
        lat.set_particles(pos, radius=4.0, rho_ratio=2.0)
        lat.step(20)
        lat.save_flow(tmp_path / "f", 1, [20, 0, 0])
        lat.save_part(tmp_path / "p")
        n0 = lat.particle_counts()[0]
        lat.step(10)
        ref = lat.particles()
    with pkg.Lattice(run) as lat:
        lat.load_flow(tmp_path / "f", 1)
        lat.load_part(tmp_path / "p", radius=4.0, rho_ratio=2.0)
        assert lat.particle_counts()[0] == n0
        lat.save_part(tmp_path / "p2")
        lat.step(10)
        got = lat.particles()
    a, b = records(tmp_path / "p"), records(tmp_path / "p2")
    assert a == b
    for k in ("pos", "vel", "omg", "force", "torque"):
        assert rel(got[k], ref[k]) < 1e-10, k


def test_driver_sphere_run_equals_binding(pkg, driver, tmp_path):
    steps = 30
    out = tmp_path / "drv"
    log = run_driver(driver, out, steps=steps, ndiag=10, nstat=30, ndiss=15, save=1, **COMMON)
    assert "spheres: 3" in log
    nx, ny, nz = SHAPE
    force = COMMON["ustar"] ** 2 / COMMON["h"]
    run = pkg.RunParams(nx=nx, ny=ny, nz=nz, visc=COMMON["visc"], force_y=force, mrt_type=1,
                        precision=pkg.PRECISIONS["fp64"])
    pos = pkg.place_spheres(nx, ny, nz, 3, 4.0, gap=2.0, wall_gap=1.0, seed=7)
    with pkg.Lattice(run) as lat:
        lat.init_channel(COMMON["uc"], COMMON["amp"], COMMON["seed"])
        lat.set_particles(pos, radius=4.0, rho_ratio=2.0)
        lat.step(steps)
        lat.save_flow(tmp_path / "api.flow", 1, [steps, 0, 0])
        st = lat.particles()
        fp, tp = lat.particle_history()
        nsolid = lat.particle_counts()[0]
    drv_flow = out / f"endrunflow2D16x8.{steps:07d}.000"
    assert records(drv_flow)[0] == records(tmp_path / "api.flow")[0]
    assert rel(flow(drv_flow), flow(tmp_path / "api.flow")) < 1e-12
    ps = part_state(out / f"endrunpart2D.{steps:07d}.000", 3)
    for k in ("pos", "vel", "omg"):
        assert rel(ps[k], st[k]) < 1e-10, k
    assert rel(ps["fprev"], fp) < 1e-10 and rel(ps["tprev"], tp) < 1e-10
    mass = 2.0 * 4.0 / 3.0 * np.pi * 4.0 ** 3
    assert rel(ps["dwdt"], fp / mass) < 1e-10 and rel(ps["domgdt"], tp / (0.4 * mass * 16.0)) < 1e-10
    check_node_flags(ps, nsolid)
    # diag.dat: one row per ndiag steps, 14 columns, solid fraction > 0
    rows = [ln.split() for ln in (out / "diag.dat").read_text().splitlines() if ln.strip()]
    assert [float(r[0]) for r in rows] == [10.0, 20.0, 30.0]
    assert all(len(r) == 14 for r in rows)
    solid = 3 * 4.0 / 3.0 * np.pi * 4.0 ** 3 / (nx * ny * nz)
    assert abs(float(rows[-1][11]) - solid) < 0.3 * solid
    # profiles2.dat: step line then nx rows of 15 columns
    prof = (out / "profiles2.dat").read_text().splitlines()
    assert prof[0].split() == ["30"] and len(prof) == 1 + nx
    assert all(len(ln.split()) == 15 for ln in prof[1:])
    # dissipation.dat: two blocks (steps 15, 30) of nx rows of 6 columns
    dis = (out / "dissipation.dat").read_text().splitlines()
    assert len(dis) == 2 * (1 + nx) and dis[0].split() == ["15"] and dis[1 + nx].split() == ["30"]
    rows = np.array([[float(v) for v in ln.split()] for ln in dis[2 + nx:]])
    assert rows.shape == (nx, 6) and (rows[:, 2] > 0).all() and (rows[:, 3] > 0).all()


def test_driver_restart_continues_sphere_run(driver, tmp_path):
    """Stop at odd step 51 and continue to 130: the restart keeps the absolute
    step (mean density removed at step 100) and the force history."""
    full, first, second = tmp_path / "full", tmp_path / "a", tmp_path / "b"
    run_driver(driver, full, steps=130, ndiag=1000, nstat=1000, save=1, **COMMON)
    run_driver(driver, first, steps=51, ndiag=1000, nstat=1000, save=1, **COMMON)
    log = run_driver(driver, second, steps=79, ndiag=1000, nstat=1000, save=1,
                     restart=first / "endrunflow2D16x8.0000051.000",
                     restart_part=first / "endrunpart2D.0000051.000", **COMMON)
    assert "istep0=51" in log
    a = flow(full / "endrunflow2D16x8.0000130.000")
    b = flow(second / "endrunflow2D16x8.0000130.000")
    assert rel(b, a) < 1e-11
    pa = part_state(full / "endrunpart2D.0000130.000", 3)
    pb = part_state(second / "endrunpart2D.0000130.000", 3)
    for k in ("pos", "vel", "omg", "fprev", "tprev"):
        assert rel(pb[k], pa[k]) < 1e-10, k
    assert np.array_equal(pa["isnodes"], pb["isnodes"])
