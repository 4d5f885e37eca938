"""ctypes binding of the FP64 CPU oracle -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
use this module, and only as the checker.  The product library and package
never import it.  Parity status: see ``lbm_oracle.h`` (pinned by the
reference's analytic Poiseuille series and by swap == push self-consistency;
no executed-reference vectors exist because the Fortran reference cannot be
built here).
"""
from __future__ import annotations

import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liblbm_oracle.so"
CFLAGS = ["-O2", "-std=c11", "-ffp-contract=off", "-fopenmp", "-fPIC", "-Wall", "-Wextra"]

Q = 19
CX = np.array([0, 1, -1, 0, 0, 0, 0, 1, -1, 1, -1, 1, -1, 1, -1, 0, 0, 0, 0])
CY = np.array([0, 0, 0, 1, -1, 0, 0, 1, 1, -1, -1, 0, 0, 0, 0, 1, -1, 1, -1])
CZ = np.array([0, 0, 0, 0, 0, 1, -1, 0, 0, 0, 0, 1, 1, -1, -1, 1, 1, -1, -1])
OPP = np.array([0, 2, 1, 4, 3, 6, 5, 10, 9, 8, 7, 14, 13, 12, 11, 18, 17, 16, 15])
W = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)


def build(force: bool = False) -> Path:
    src = [HERE / "lbm_oracle.c", HERE / "lbm_oracle.h"]
    if force or not LIB.exists() or any(s.stat().st_mtime > LIB.stat().st_mtime for s in src):
        LIB.parent.mkdir(exist_ok=True)
        cc = shutil.which("gcc") or "gcc"
        tmp = LIB.with_suffix(".tmp")
        subprocess.run([cc, *CFLAGS, "-shared", "-o", str(tmp), str(HERE / "lbm_oracle.c"), "-lm"], check=True)
        tmp.replace(LIB)
    return LIB


class OrcParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("s1", "s2", "s4", "s9", "s10", "s13", "s16",
                                               "omegepsl", "omegepslj", "omegxx")] + \
               [("force", ctypes.c_double * 3)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB))
        dp = ctypes.POINTER(ctypes.c_double)
        pp = ctypes.POINTER(OrcParams)
        i = ctypes.c_int
        sig = {
            "orc_collide_node": (None, [pp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, dp]),
            "orc_force_moments": (None, [pp, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp]),
            "orc_moment_row": (None, [i, ctypes.POINTER(ctypes.c_int), dp]),
            "orc_macrovar": (None, [pp, dp, i, i, i, dp, dp, dp, dp]),
            "orc_initpop": (None, [i, i, i, dp, dp, dp, dp]),
            "orc_rhoupdat": (None, [dp, i, i, i, dp]),
            "orc_step_swap": (i, [pp, dp, i, i, i, dp, dp, dp, dp]),
            "orc_step_push": (None, [pp, dp, dp, i, i, i, dp, dp, dp, dp]),
            "orc_run": (i, [pp, dp, i, i, i, i, i, dp, dp, dp, dp]),
            "orc_prerelax": (i, [pp, dp, i, i, i, dp, dp, dp, ctypes.c_double, i, ctypes.POINTER(i), dp]),
            "orc_run_omp": (i, [pp, dp, i, i, i, i, i]),
            "orc_max_threads": (i, []),
            "orc_profiles": (None, [dp, dp, dp, dp, i, i, i, dp]),
            "orc_channel_velocity": (None, [i, i, i, ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                            dp, dp, dp]),
            "orc_loglaw_velocity": (None, [i, i, i, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp, dp, dp]),
            "orc_particles_place": (i, [i, i, i, i, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_uint64, dp]),
        }
        for name, (res, args) in sig.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def params(rates: dict, force=(0.0, 0.0, 0.0)) -> OrcParams:
    p = OrcParams()
    for k in ("s1", "s2", "s4", "s9", "s10", "s13", "s16", "omegepsl", "omegepslj", "omegxx"):
        setattr(p, k, rates[k])
    p.force[:] = list(force)
    return p


def params_from(run) -> OrcParams:
    """Oracle parameters from a package RunParams."""
    return params(run.rates(), (0.0, run.force_y, 0.0))


def fields(shape):
    return [np.zeros(shape, dtype=np.float64, order="F") for _ in range(4)]


def collide_node(p: OrcParams, f, rho, ux, uy, uz) -> np.ndarray:
    f = np.ascontiguousarray(f, dtype=np.float64)
    out = np.empty(Q)
    lib().orc_collide_node(ctypes.byref(p), _p(f), rho, ux, uy, uz, _p(out))
    return out


def force_moments(p: OrcParams, ux, uy, uz) -> np.ndarray:
    out = np.empty(Q)
    lib().orc_force_moments(ctypes.byref(p), ux, uy, uz, _p(out))
    return out


def moment_matrix() -> tuple[np.ndarray, np.ndarray]:
    M = np.zeros((Q, Q), dtype=np.int64)
    d = np.zeros(Q)
    row = (ctypes.c_int * Q)()
    n2 = ctypes.c_double()
    for k in range(Q):
        lib().orc_moment_row(k, row, ctypes.byref(n2))
        M[k] = list(row)
        d[k] = n2.value
    return M, d


def macrovar(p: OrcParams, f: np.ndarray):
    _, nx, ny, nz = f.shape
    out = fields((nx, ny, nz))
    lib().orc_macrovar(ctypes.byref(p), _p(f), nx, ny, nz, *map(_p, out))
    return tuple(out)


def initpop(ux, uy, uz) -> np.ndarray:
    nx, ny, nz = ux.shape
    f = np.empty((Q, nx, ny, nz), dtype=np.float64, order="F")
    a, b, c = (np.asfortranarray(v, dtype=np.float64) for v in (ux, uy, uz))
    lib().orc_initpop(nx, ny, nz, _p(a), _p(b), _p(c), _p(f))
    return f


def run(p: OrcParams, f: np.ndarray, nsteps: int, mode: int = 0):
    """main.f90:136-161 on a copy of f; returns (f, rho, ux, uy, uz)."""
    f = np.array(f, dtype=np.float64, order="F", copy=True)
    _, nx, ny, nz = f.shape
    out = fields((nx, ny, nz))
    rc = lib().orc_run(ctypes.byref(p), _p(f), nx, ny, nz, nsteps, mode, *map(_p, out))
    if rc != 0:
        raise RuntimeError("oracle run failed")
    return (f, *out)


def step_swap(p: OrcParams, f: np.ndarray, rho, ux, uy, uz) -> np.ndarray:
    f = np.array(f, dtype=np.float64, order="F", copy=True)
    _, nx, ny, nz = f.shape
    m = [np.asfortranarray(v, dtype=np.float64) for v in (rho, ux, uy, uz)]
    if lib().orc_step_swap(ctypes.byref(p), _p(f), nx, ny, nz, *map(_p, m)) != 0:
        raise RuntimeError("oracle swap failed")
    return f


def step_push(p: OrcParams, f: np.ndarray, rho, ux, uy, uz) -> np.ndarray:
    f = np.asfortranarray(f, dtype=np.float64)
    _, nx, ny, nz = f.shape
    g = np.empty_like(f, order="F")
    m = [np.asfortranarray(v, dtype=np.float64) for v in (rho, ux, uy, uz)]
    lib().orc_step_push(ctypes.byref(p), _p(f), _p(g), nx, ny, nz, *map(_p, m))
    return g


def prerelax(p: OrcParams, f: np.ndarray, ux, uy, uz, eps=1e-5, maxit=15000):
    f = np.array(f, dtype=np.float64, order="F", copy=True)
    _, nx, ny, nz = f.shape
    it = ctypes.c_int()
    err = ctypes.c_double()
    a, b, c = (np.asfortranarray(v, dtype=np.float64) for v in (ux, uy, uz))
    rc = lib().orc_prerelax(ctypes.byref(p), _p(f), nx, ny, nz, _p(a), _p(b), _p(c), eps, maxit,
                            ctypes.byref(it), ctypes.byref(err))
    if rc < 0:
        raise RuntimeError("oracle prerelax failed")
    return f, it.value, err.value, rc


def run_omp(p: OrcParams, f: np.ndarray, nsteps: int, nthreads: int) -> np.ndarray:
    _, nx, ny, nz = f.shape
    if lib().orc_run_omp(ctypes.byref(p), _p(f), nx, ny, nz, nsteps, nthreads) != 0:
        raise RuntimeError("oracle omp run failed")
    return f


def max_threads() -> int:
    return lib().orc_max_threads()


def profiles(rho, ux, uy, uz) -> np.ndarray:
    nx, ny, nz = rho.shape
    out = np.empty((nx, 12))
    m = [np.asfortranarray(v, dtype=np.float64) for v in (rho, ux, uy, uz)]
    lib().orc_profiles(*map(_p, m), nx, ny, nz, _p(out))
    return out


def channel_velocity(nx, ny, nz, uc, amp, seed):
    out = [np.empty((nx, ny, nz), dtype=np.float64, order="F") for _ in range(3)]
    lib().orc_channel_velocity(nx, ny, nz, uc, amp, ctypes.c_uint64(seed), *map(_p, out))
    return tuple(out)


def loglaw_velocity(nx, ny, nz, ustar, ystar, a9=0.0):
    """initvel's turbulent start (initial.f90:101-147), reference layout."""
    out = [np.empty((nx, ny, nz), dtype=np.float64, order="F") for _ in range(3)]
    lib().orc_loglaw_velocity(nx, ny, nz, ustar, ystar, a9, *map(_p, out))
    return tuple(out)


def place_spheres(nx, ny, nz, npart, radius, gap=2.0, wall_gap=1.0, seed=12345) -> np.ndarray:
    """Seeded non-overlapping sphere centres (reference axes), shape (npart, 3)."""
    pos = np.empty((npart, 3), dtype=np.float64)
    rc = lib().orc_particles_place(nx, ny, nz, npart, radius, gap, wall_gap, ctypes.c_uint64(seed), _p(pos))
    if rc != 0:
        raise ValueError("could not place all spheres (volume fraction too high)")
    return pos


def poiseuille_transient(nx: int, ustar: float, visc: float, istep: int, nterms: int = 26) -> np.ndarray:
    """Analytic laminar start-up profile u(x)/ustar at the nodes of the lower
    half, the series outputuy writes (saveload.f90:921-933)."""
    time1 = istep * visc / (nx / 2.0) ** 2
    i = np.arange(1, nx // 2 + 1)
    xx0 = np.abs(i - 0.5 - nx / 2.0)
    s = np.zeros_like(xx0)
    for n in range(nterms):
        s += (4 * (-1) ** n) / (np.pi * (n + 0.5)) ** 3 * np.exp(-((n + 0.5) ** 2) * np.pi**2 * time1) * \
            np.cos((n + 0.5) * np.pi * (xx0 / (nx / 2.0)))
    return (1 - (xx0 / (nx / 2.0)) ** 2) - s


# ---- moving spheres --------------------------------------------------------
class OrcParticles(ctypes.Structure):
    _fields_ = [("npart", ctypes.c_int), ("radius", ctypes.c_double), ("rho_ratio", ctypes.c_double),
                ("stf0", ctypes.c_double), ("stf1", ctypes.c_double), ("stf0_w", ctypes.c_double),
                ("stf1_w", ctypes.c_double), ("zeta", ctypes.c_double)] + \
               [(n, ctypes.POINTER(ctypes.c_double)) for n in
                ("pos", "vel", "omg", "force", "torque", "force_prev", "torque_prev")] + \
               [("have_prev", ctypes.c_int)]


class Spheres:
    """Sphere state for the oracle; arrays (npart, 3) float64, reference axes."""

    def __init__(self, pos, radius, rho_ratio=2.0, vel=None, omg=None, stf0=0.025, stf1=0.002,
                 stf0_w=0.025, stf1_w=0.002, zeta=1.0):
        self.pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3).copy()
        n = len(self.pos)
        self.vel = np.zeros((n, 3)) if vel is None else np.array(vel, dtype=np.float64).reshape(n, 3)
        self.omg = np.zeros((n, 3)) if omg is None else np.array(omg, dtype=np.float64).reshape(n, 3)
        self.force = np.zeros((n, 3))
        self.torque = np.zeros((n, 3))
        self.force_prev = np.zeros((n, 3))
        self.torque_prev = np.zeros((n, 3))
        self.c = OrcParticles()
        self.c.npart = n
        self.c.radius = radius
        self.c.rho_ratio = rho_ratio
        self.c.stf0, self.c.stf1, self.c.stf0_w, self.c.stf1_w, self.c.zeta = stf0, stf1, stf0_w, stf1_w, zeta
        for name in ("pos", "vel", "omg", "force", "torque", "force_prev", "torque_prev"):
            setattr(self.c, name, _p(getattr(self, name)))
        self.c.have_prev = 0


def _bind_particles():
    L = lib()
    if getattr(L, "_particles_bound", False):
        return L
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    L.orc_mark_solid.restype = None
    L.orc_mark_solid.argtypes = [ctypes.POINTER(OrcParticles), ctypes.c_int, ctypes.c_int, ctypes.c_int, ip]
    L.orc_particle_step.restype = ctypes.c_int
    L.orc_particle_step.argtypes = [ctypes.POINTER(OrcParams), ctypes.POINTER(OrcParticles), dp, ctypes.c_int,
                                    ctypes.c_int, ctypes.c_int, ip, ip, ip]
    L._particles_bound = True
    return L


def mark_solid(sp: Spheres, shape) -> np.ndarray:
    L = _bind_particles()
    owner = np.empty(shape, dtype=np.int32, order="F")
    L.orc_mark_solid(ctypes.byref(sp.c), *shape, owner.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    return owner


def particle_run(p: OrcParams, sp: Spheres, f: np.ndarray, nsteps: int, owner=None):
    """nsteps particle-laden steps in place on a copy of f; returns (f, owner, links, refills)."""
    L = _bind_particles()
    f = np.array(f, dtype=np.float64, order="F", copy=True)
    _, nx, ny, nz = f.shape
    if owner is None:
        owner = mark_solid(sp, (nx, ny, nz))
    ip = ctypes.POINTER(ctypes.c_int)
    nl, nr = ctypes.c_int(), ctypes.c_int()
    links, refills = [], []
    for _ in range(nsteps):
        rc = L.orc_particle_step(ctypes.byref(p), ctypes.byref(sp.c), _p(f), nx, ny, nz,
                                 owner.ctypes.data_as(ip), ctypes.byref(nl), ctypes.byref(nr))
        if rc != 0:
            raise RuntimeError("oracle particle step failed")
        links.append(nl.value)
        refills.append(nr.value)
    return f, owner, links, refills


# ---- strain rate from the non-equilibrium populations (sijstat01) -----------
def strain_sij2(p: OrcParams, f: np.ndarray, s1: float, s9: float):
    """S_ij S_ij per node by the two methods of sijstat01, in FP64, written
    with the reference's own sums (saveload.f90:2322-2380, population order
    of para.f90) so that it checks the GPU's lattice-vector formulation:
    method 1 from the non-equilibrium moments (Yu et al. 2006), method 2 from
    f - f^eq (saveload.f90:2385-2432).  f: (19, nx, ny, nz) deviations."""
    rho, ux, uy, uz = macrovar(p, f)
    ux2, uy2, uz2 = ux * ux, uy * uy, uz * uz
    eqm1 = -11.0 * rho + 19.0 * (ux2 + uy2 + uz2)           # :2337-2342
    eqm6 = 2.0 * ux2 - uy2 - uz2
    eqm8 = uy2 - uz2
    eqm10, eqm11, eqm12 = ux * uy, uy * uz, ux * uz
    sum1 = f[1:7].sum(axis=0)                                # :2344-2355
    sum2 = f[7:19].sum(axis=0)
    sum6 = f[1] + f[2]
    sum7 = f[3] + f[4] + f[5] + f[6]
    sum8 = f[7:15].sum(axis=0)
    sum9 = f[15:19].sum(axis=0)
    sum10 = f[3] + f[4] - f[5] - f[6]
    sum11 = f[7] + f[8] + f[9] + f[10] - f[11] - f[12] - f[13] - f[14]
    evlm1 = -30.0 * f[0] - 11.0 * sum1 + 8.0 * sum2          # :2357-2362 (coef2, coef3, coef5)
    evlm6 = 2.0 * sum6 - sum7 + sum8 - 2.0 * sum9
    evlm8 = sum10 + sum11
    evlm10 = f[7] - f[8] - f[9] + f[10]
    evlm11 = f[15] - f[16] - f[17] + f[18]
    evlm12 = f[11] - f[12] - f[13] + f[14]
    n1 = s1 * (evlm1 - eqm1)                                 # :2364-2369
    n9 = s9 * (evlm6 - eqm6)
    n11 = s9 * (evlm8 - eqm8)
    n13 = s9 * (evlm10 - eqm10)
    n14 = s9 * (evlm11 - eqm11)
    n15 = s9 * (evlm12 - eqm12)
    sxx = -(n1 + 19.0 * n9) / 38.0                           # :2371-2376
    syy = -(2.0 * n1 - 19.0 * (n9 - 3.0 * n11)) / 76.0
    szz = -(2.0 * n1 - 19.0 * (n9 + 3.0 * n11)) / 76.0
    sxy, syz, szx = -1.5 * n13, -1.5 * n14, -1.5 * n15
    m1 = sxx**2 + syy**2 + szz**2 + 2.0 * (sxy**2 + syz**2 + szx**2)
    usqr = 1.5 * (ux2 + uy2 + uz2)                            # :2385-2397
    a = np.zeros((6,) + rho.shape)
    for i in range(1, Q):
        cu = CX[i] * ux + CY[i] * uy + CZ[i] * uz
        fn = f[i] - W[i] * (rho + 3.0 * cu + 4.5 * cu * cu - usqr)
        a[0] += fn * CX[i] * CX[i]
        a[1] += fn * CY[i] * CY[i]
        a[2] += fn * CZ[i] * CZ[i]
        a[3] += fn * CX[i] * CY[i]
        a[4] += fn * CY[i] * CZ[i]
        a[5] += fn * CZ[i] * CX[i]
    m2 = (a[0]**2 + a[1]**2 + a[2]**2 + 2.0 * (a[3]**2 + a[4]**2 + a[5]**2)) * (1.5 * s9) ** 2
    return m1, m2


def dissipation_sums(p: OrcParams, f: np.ndarray, s1: float, s9: float, solid=None):
    """dissipation_calc (saveload.f90:4644-4882): per wall-normal plane the
    sums over fluid nodes of S_ij S_ij (moments, f - f^eq) and S_xy of both
    methods, and the fluid count; (nx, 5).  S_xy: -1.5 neqm13 (:4730) and
    (1.5 / tau) sum fneq c_x c_y (:4772).  solid: (nx, ny, nz) bool or None."""
    m1, m2 = strain_sij2(p, f, s1, s9)
    rho, ux, uy, uz = macrovar(p, f)
    sxy1 = strain_tensor(p, f, s1, s9)[3]
    usqr = 1.5 * (ux * ux + uy * uy + uz * uz)
    a = np.zeros_like(rho)
    for i in range(1, Q):
        cu = CX[i] * ux + CY[i] * uy + CZ[i] * uz
        a += (f[i] - W[i] * (rho + 3.0 * cu + 4.5 * cu * cu - usqr)) * CX[i] * CY[i]
    sxy2 = a * (1.5 * s9)
    fluid = np.ones_like(m1, dtype=bool) if solid is None else ~solid
    out = np.empty((m1.shape[0], 5))
    for k, v in enumerate((m1, m2, sxy1, sxy2)):
        out[:, k] = np.where(fluid, v, 0.0).sum(axis=(1, 2))
    out[:, 4] = fluid.sum(axis=(1, 2))
    return out


# ---- learned LES closure network (no reference counterpart) -----------------
MLP_IN, MLP_H = 7, 32
MLP_PARAMS = MLP_IN * MLP_H + MLP_H + MLP_H * MLP_H + MLP_H + MLP_H + 1


def mlp_unpack(p):
    """(W1[7][32], b1, W2[32][32], b2, w3, b3) views of the parameter vector,
    in the C ABI's order (W rows are inputs)."""
    p = np.asarray(p, dtype=np.float64)
    o = 0
    W1 = p[o:o + MLP_IN * MLP_H].reshape(MLP_IN, MLP_H); o += MLP_IN * MLP_H
    b1 = p[o:o + MLP_H]; o += MLP_H
    W2 = p[o:o + MLP_H * MLP_H].reshape(MLP_H, MLP_H); o += MLP_H * MLP_H
    b2 = p[o:o + MLP_H]; o += MLP_H
    w3 = p[o:o + MLP_H]; o += MLP_H
    return W1, b1, W2, b2, w3, p[o]


def _sigmoid(x):
    return 1.0 / (1.0 + np.exp(-x))


def mlp_forward(p, norm, X):
    """nu_t / nu for raw features X[n][7] in FP64 (the network of lbm_mlp.cuh)."""
    W1, b1, W2, b2, w3, b3 = mlp_unpack(p)
    norm = np.asarray(norm, dtype=np.float64)
    xn = (np.asarray(X, dtype=np.float64) - norm[:MLP_IN]) * norm[MLP_IN:]
    z1 = xn @ W1 + b1
    h1 = z1 * _sigmoid(z1)
    z2 = h1 @ W2 + b2
    h2 = z2 * _sigmoid(z2)
    z3 = h2 @ w3 + b3
    return np.where(z3 > 20.0, z3, np.log1p(np.exp(np.minimum(z3, 20.0)))), (xn, z1, h1, z2, h2, z3)


def mlp_loss_grad(p, norm, X, y):
    """Mean squared error of nu_t / nu and its analytic gradient, FP64."""
    out, (xn, z1, h1, z2, h2, z3) = mlp_forward(p, norm, X)
    W1, b1, W2, b2, w3, b3 = mlp_unpack(p)
    n = len(y)
    diff = out - np.asarray(y, dtype=np.float64)
    loss = float(np.mean(diff * diff))
    dz3 = 2.0 * diff * _sigmoid(z3) / n
    dsilu = lambda z: _sigmoid(z) * (1.0 + z * (1.0 - _sigmoid(z)))
    dw3 = h2.T @ dz3
    db3 = dz3.sum()
    dz2 = np.outer(dz3, w3) * dsilu(z2)
    dW2 = h1.T @ dz2
    db2 = dz2.sum(axis=0)
    dz1 = (dz2 @ W2.T) * dsilu(z1)
    dW1 = xn.T @ dz1
    db1 = dz1.sum(axis=0)
    g = np.concatenate([dW1.ravel(), db1, dW2.ravel(), db2, dw3, [db3]])
    return loss, g


def mlp_adam(p, g, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) on FP64 copies; returns (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    p = p - lr * (m / (1 - b1**t)) / (np.sqrt(v / (1 - b2**t)) + eps)
    return p, m, v


def strain_tensor(p: OrcParams, f: np.ndarray, s1: float, s9):
    """S = {xx, yy, zz, xy, yz, zx} per node from the non-equilibrium moments
    (the same formulas as strain_sij2's method 1, saveload.f90:2322-2376);
    s9 may be a per-node array (the shear rate that produced the
    non-equilibrium part)."""
    rho, ux, uy, uz = macrovar(p, f)
    ux2, uy2, uz2 = ux * ux, uy * uy, uz * uz
    sum1 = f[1:7].sum(axis=0)
    sum2 = f[7:19].sum(axis=0)
    evlm1 = -30.0 * f[0] - 11.0 * sum1 + 8.0 * sum2
    evlm6 = 2.0 * (f[1] + f[2]) - (f[3] + f[4] + f[5] + f[6]) + f[7:15].sum(axis=0) - 2.0 * f[15:19].sum(axis=0)
    evlm8 = (f[3] + f[4] - f[5] - f[6]) + (f[7] + f[8] + f[9] + f[10] - f[11] - f[12] - f[13] - f[14])
    n1 = s1 * (evlm1 - (-11.0 * rho + 19.0 * (ux2 + uy2 + uz2)))
    n9 = s9 * (evlm6 - (2.0 * ux2 - uy2 - uz2))
    n11 = s9 * (evlm8 - (uy2 - uz2))
    S = np.empty((6,) + rho.shape)
    S[0] = -(n1 + 19.0 * n9) / 38.0
    S[1] = -(2.0 * n1 - 19.0 * (n9 - 3.0 * n11)) / 76.0
    S[2] = -(2.0 * n1 - 19.0 * (n9 + 3.0 * n11)) / 76.0
    S[3] = -1.5 * s9 * (f[7] - f[8] - f[9] + f[10] - ux * uy)
    S[4] = -1.5 * s9 * (f[15] - f[16] - f[17] + f[18] - uy * uz)
    S[5] = -1.5 * s9 * (f[11] - f[12] - f[13] + f[14] - ux * uz)
    return S


def closure_features(S, dwall, nu, ustar, h):
    """The closure's 7 inputs (as lbm_mlp.cuh) in FP64; S (6, ...) and dwall
    broadcastable; returns (..., 7)."""
    tr = S[0] + S[1] + S[2]
    off = S[3] ** 2 + S[4] ** 2 + S[5] ** 2
    smag = np.sqrt(2.0 * (S[0] ** 2 + S[1] ** 2 + S[2] ** 2 + 2.0 * off))
    d0, d1, d2 = S[0] - tr / 3, S[1] - tr / 3, S[2] - tr / 3
    rn = np.sqrt(d0 * d0 + d1 * d1 + d2 * d2 + 2.0 * off) + 1e-30
    det = d0 * (d1 * d2 - S[4] ** 2) - S[3] * (S[3] * d2 - S[4] * S[5]) + S[5] * (S[3] * S[4] - d1 * S[5])
    dwall = np.broadcast_to(dwall, tr.shape)
    return np.stack([np.log1p(smag * nu / ustar**2), tr / (smag + 1e-30), np.sqrt(6.0) * det / rn**3,
                     d0 / rn, np.sqrt(S[3] ** 2 + S[5] ** 2) / rn, np.log1p(dwall * ustar / nu),
                     dwall / h], axis=-1)


OPP = np.array([int(np.flatnonzero((CX == -CX[i]) & (CY == -CY[i]) & (CZ == -CZ[i]))[0]) for i in range(Q)])


def les_step(p: OrcParams, f: np.ndarray, s9prev: np.ndarray, params, norm, ustar: float, h: float,
             aplus: float = 0.0):
    """One coarse-LES step with the closure, FP64: per node the strain from the
    non-equilibrium moments with s9prev, the features and the network give
    s9 = s13 = 1/(3 nu (1 + nu_t/nu) + 1/2); collide_node with those rates;
    push streaming with half-way bounce-back at the x walls and periodic y, z.
    Returns (f, s9).  Small lattices only (a Python loop over nodes)."""
    _, nx, ny, nz = f.shape
    nu = (1.0 / p.s9 - 0.5) / 3.0
    S = strain_tensor(p, f, p.s1, s9prev)
    dwall = np.minimum(np.arange(nx) + 0.5, nx - np.arange(nx) - 0.5)[:, None, None]
    X = closure_features(S, dwall, nu, ustar, h).reshape(-1, 7)
    r, _ = mlp_forward(params, norm, X)
    if aplus > 0.0:                      # van Driest damping of nu_t
        yp = np.broadcast_to(dwall * ustar / nu, (nx, ny, nz)).reshape(-1)
        r = r * (1.0 - np.exp(-yp / aplus)) ** 2
    s9 = (1.0 / (3.0 * nu * (1.0 + r) + 0.5)).reshape(nx, ny, nz)
    rho, ux, uy, uz = macrovar(p, f)
    post = np.empty_like(f)
    q = OrcParams.from_buffer_copy(p)
    for ix in range(nx):
        for iy in range(ny):
            for iz in range(nz):
                q.s9 = q.s13 = s9[ix, iy, iz]
                post[:, ix, iy, iz] = collide_node(q, np.ascontiguousarray(f[:, ix, iy, iz]), rho[ix, iy, iz],
                                                   ux[ix, iy, iz], uy[ix, iy, iz], uz[ix, iy, iz])
    out = np.empty_like(f)
    for i in range(Q):
        moved = np.roll(np.roll(post[i], CY[i], axis=1), CZ[i], axis=2)
        if CX[i] == 0:
            out[i] = moved
        elif CX[i] > 0:
            out[i, 1:] = moved[:-1]
        else:
            out[i, :-1] = moved[1:]
    # half-way bounce-back: a population leaving through a wall comes back
    # into the opposite direction at the same node
    for i in range(Q):
        if CX[i] > 0:
            out[OPP[i], -1] = post[i, -1]
        elif CX[i] < 0:
            out[OPP[i], 0] = post[i, 0]
    return out, s9


def closure_training_data(p: OrcParams, f: np.ndarray, factor: int, ustar: float, h: float):
    """Box filter by `factor`, strain of the filtered velocity by central
    differences (periodic y, z; no-slip image across the x walls), closure
    features (coarse units: nu/factor, h/factor) and the target
    max(0, -tau^d:S / (2 S:S)) / nu_c, FP64.  Returns (X[nc][7], y[nc],
    ubar[3][nxc][nyc][nzc]) with coarse cells in Fortran order."""
    _, ux, uy, uz = macrovar(p, f)
    nx, ny, nz = ux.shape
    nxc, nyc, nzc = nx // factor, ny // factor, nz // factor

    def box(a):
        return a.reshape(nxc, factor, nyc, factor, nzc, factor).mean(axis=(1, 3, 5))

    u = [box(ux), box(uy), box(uz)]
    uu = {(a, b): box([ux, uy, uz][a] * [ux, uy, uz][b]) for a in range(3) for b in range(a, 3)}

    def grad(v):
        g = np.empty((3,) + v.shape)
        ext = np.concatenate([-v[:1], v, -v[-1:]], axis=0)           # no-slip image
        g[0] = 0.5 * (ext[2:] - ext[:-2])
        g[1] = 0.5 * (np.roll(v, -1, axis=1) - np.roll(v, 1, axis=1))
        g[2] = 0.5 * (np.roll(v, -1, axis=2) - np.roll(v, 1, axis=2))
        return g

    G = [grad(v) for v in u]                                          # G[a][b] = d u_a / d x_b
    S = np.stack([G[0][0], G[1][1], G[2][2], 0.5 * (G[0][1] + G[1][0]), 0.5 * (G[1][2] + G[2][1]),
                  0.5 * (G[0][2] + G[2][0])])
    tau = np.stack([uu[(0, 0)] - u[0] ** 2, uu[(1, 1)] - u[1] ** 2, uu[(2, 2)] - u[2] ** 2,
                    uu[(0, 1)] - u[0] * u[1], uu[(1, 2)] - u[1] * u[2], uu[(0, 2)] - u[0] * u[2]])
    t3 = (tau[0] + tau[1] + tau[2]) / 3.0
    tau[:3] -= t3
    num = -(tau[0] * S[0] + tau[1] * S[1] + tau[2] * S[2] + 2.0 * (tau[3] * S[3] + tau[4] * S[4] + tau[5] * S[5]))
    den = 2.0 * (S[0] ** 2 + S[1] ** 2 + S[2] ** 2 + 2.0 * (S[3] ** 2 + S[4] ** 2 + S[5] ** 2))
    nut = np.where(den > 0, np.maximum(num / np.where(den > 0, den, 1.0), 0.0), 0.0)
    nu_c = (1.0 / p.s9 - 0.5) / 3.0 / factor
    dwall = np.minimum(np.arange(nxc) + 0.5, nxc - np.arange(nxc) - 0.5)[:, None, None]
    X = closure_features(S, dwall, nu_c, ustar, h / factor)
    X = np.stack([X[..., k].ravel(order="F") for k in range(7)], axis=1)
    return X, (nut / nu_c).ravel(order="F"), np.stack(u)
