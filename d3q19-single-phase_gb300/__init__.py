"""GB300-native D3Q19 channel-flow time step (host-side Python mirror).

This package is a thin ctypes layer over ``liblbm_gb300.so``, whose
``extern "C"`` boundary is declared in ``include/lbm_gb300.h``.  It mirrors the
reference's drop-in interface for the hot path:

* :func:`para` restates the run constants of ``Channel-Flow/para.f90:59-141``
  (laminar/turbulent channel, MRT rate sets) for a lattice of any size;
* :class:`Lattice` owns the device state and exposes the reference's
  subroutines as methods -- ``initpop`` (initial.f90:19-46), ``step``
  (collision_MRT + collisionExchnge + macrovar, collision.f90:24-463),
  ``prerelax`` (main.f90:69-90), ``macrovar``, ``diag`` and ``profiles``
  (saveload.f90:1202-1676), ``save_flow``/``load_flow`` (saveload.f90:102-332);
* ``Lattice.set_particles``/``particles``: moving solid spheres (interpolated
  bounce-back, momentum exchange, refilling, Newton-Euler) run after every
  step; the reference declares their data (var_inc.f90:120-150) without the
  algorithm, which is this project's own;
* ``Lattice.strain``: S_ij S_ij from the non-equilibrium populations, both
  methods of sijstat01 (saveload.f90:2320-2432);
* :class:`ClosureNet` and ``Lattice.les_set``/``les_training_data``: the
  learned LES closure (no reference counterpart) -- a per-node eddy-viscosity
  network trained on the GPU on box-filtered DNS and fused into the collision
  of a coarse-grid LES; ``les_closure.py`` runs it end to end;
* :data:`CHANNEL_CONFIGS` holds the benchmark channel workloads.

Arrays use the reference layout: populations ``f(0:18, nx, ny, nz)`` and
fields ``(nx, ny, nz)``, Fortran order, float64; x is wall-normal, y
streamwise, z spanwise.

There is no CPU fallback: importing works without a GPU, but creating a
:class:`Lattice` needs the built library and a CUDA device, and raises
otherwise.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "liblbm_gb300.so"

PREC_FP64, PREC_FP32, PREC_FP16 = 0, 1, 2
PRECISIONS = {"fp64": PREC_FP64, "fp32": PREC_FP32, "fp16": PREC_FP16}
MRT_STABLE, MRT_LBGK, MRT_LOWDISS = 1, 2, 3
PROFILE_COLS = 12
DISSIPATION_COLS = 5
FLAG_SIMPLE_STEP = 1
PFLAG_Q_FP64 = 1
PROFILE_NAMES = ("ux", "uy", "uz", "uxuz", "uxuy", "uyuz", "uxux", "uyuy", "uzuz", "rho", "rhorho", "count")

# Every symbol include/lbm_gb300.h declares.
EXPORTS = (
    "lbm_strerror", "lbm_last_error", "lbm_version", "lbm_params_init", "lbm_create", "lbm_destroy",
    "lbm_device_bytes", "lbm_upload_f", "lbm_download_f", "lbm_initpop", "lbm_init_channel",
    "lbm_channel_velocity", "lbm_init_loglaw", "lbm_loglaw_velocity", "lbm_step", "lbm_step_async", "lbm_synchronize", "lbm_stream",
    "lbm_step_count", "lbm_set_step_count", "lbm_prerelax", "lbm_macrovar", "lbm_diag", "lbm_profiles", "lbm_avedensity",
    "lbm_save_flow", "lbm_load_flow", "lbm_profiles_noalloc", "lbm_particle_params_init",
    "lbm_particles_place", "lbm_particles_set", "lbm_particles_get", "lbm_particles_get_history",
    "lbm_particles_set_history", "lbm_save_part", "lbm_load_part", "lbm_particle_counts",
    "lbm_dissipation",
    "lbm_timing_enable", "lbm_timing_get", "lbm_step_launches", "lbm_strain",
    "lbm_mlp_create", "lbm_mlp_destroy", "lbm_mlp_get", "lbm_mlp_set", "lbm_mlp_set_data", "lbm_mlp_train",
    "lbm_mlp_gradient", "lbm_mlp_predict", "lbm_les_set", "lbm_les_wall_damping", "lbm_les_nut", "lbm_les_training_data",
    "lbm_les_features",
)


class LBMError(RuntimeError):
    """A negative status code returned by the C ABI."""

    def __init__(self, code: int, where: str, detail: str):
        super().__init__(f"{where}: {detail} (code {code})")
        self.code = code


class LBMParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("s1", ctypes.c_double), ("s2", ctypes.c_double), ("s4", ctypes.c_double),
        ("s9", ctypes.c_double), ("s10", ctypes.c_double), ("s13", ctypes.c_double),
        ("s16", ctypes.c_double),
        ("omegepsl", ctypes.c_double), ("omegepslj", ctypes.c_double), ("omegxx", ctypes.c_double),
        ("force", ctypes.c_double * 3),
        ("fp16_scale", ctypes.c_double),
        ("device", ctypes.c_int32), ("flags", ctypes.c_int32),
    ]


class LBMStats(ctypes.Structure):
    _fields_ = [
        ("nfluid", ctypes.c_int64), ("rho_sum", ctypes.c_double),
        ("mom_sum", ctypes.c_double * 3), ("usq_sum", ctypes.c_double * 3),
        ("rho_max", ctypes.c_double), ("rho_min", ctypes.c_double), ("vmax", ctypes.c_double),
        ("vmax_at", ctypes.c_int32 * 3), ("nonfinite", ctypes.c_int32),
    ]


class LBMParticleParams(ctypes.Structure):
    _fields_ = [("npart", ctypes.c_int32), ("flags", ctypes.c_int32), ("radius", ctypes.c_double),
                ("rho_ratio", ctypes.c_double), ("stf0", ctypes.c_double), ("stf1", ctypes.c_double),
                ("stf0_w", ctypes.c_double), ("stf1_w", ctypes.c_double), ("zeta", ctypes.c_double)]


_lib = None


def library_path() -> Path:
    return LIB_PATH


def load_library(path: Path | str | None = None) -> ctypes.CDLL:
    """Load liblbm_gb300.so (built by ``__graft_entry__.build()``); raise if absent."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(f"{p} is missing: build it with __graft_entry__.build() (needs nvcc)")
    lib = ctypes.CDLL(str(p))
    dp = ctypes.POINTER(ctypes.c_double)
    fp = ctypes.POINTER(ctypes.c_float)
    ctx = ctypes.c_void_p
    sig = {
        "lbm_strerror": (ctypes.c_char_p, [ctypes.c_int]),
        "lbm_last_error": (ctypes.c_char_p, []),
        "lbm_version": (ctypes.c_int, []),
        "lbm_params_init": (ctypes.c_int, [ctypes.POINTER(LBMParams), ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                           ctypes.c_int32]),
        "lbm_create": (ctypes.c_int, [ctypes.POINTER(LBMParams), ctypes.POINTER(ctx)]),
        "lbm_destroy": (ctypes.c_int, [ctx]),
        "lbm_device_bytes": (ctypes.c_int, [ctx, ctypes.POINTER(ctypes.c_size_t)]),
        "lbm_upload_f": (ctypes.c_int, [ctx, dp]),
        "lbm_download_f": (ctypes.c_int, [ctx, dp]),
        "lbm_initpop": (ctypes.c_int, [ctx, dp, dp, dp]),
        "lbm_init_channel": (ctypes.c_int, [ctx, ctypes.c_double, ctypes.c_double, ctypes.c_uint64]),
        "lbm_init_loglaw": (ctypes.c_int, [ctx, ctypes.c_double, ctypes.c_double, ctypes.c_double]),
        "lbm_loglaw_velocity": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                               ctypes.c_double, ctypes.c_double, dp, dp, dp]),
        "lbm_channel_velocity": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_double,
                                                ctypes.c_double, ctypes.c_uint64, dp, dp, dp]),
        "lbm_step": (ctypes.c_int, [ctx, ctypes.c_int32]),
        "lbm_step_async": (ctypes.c_int, [ctx, ctypes.c_int32]),
        "lbm_synchronize": (ctypes.c_int, [ctx]),
        "lbm_stream": (ctypes.c_int, [ctx, ctypes.POINTER(ctypes.c_void_p)]),
        "lbm_step_count": (ctypes.c_int, [ctx, ctypes.POINTER(ctypes.c_int64)]),
        "lbm_step_launches": (ctypes.c_int, [ctx, ctypes.POINTER(ctypes.c_int64)]),
        "lbm_set_step_count": (ctypes.c_int, [ctx, ctypes.c_int64]),
        "lbm_prerelax": (ctypes.c_int, [ctx, dp, dp, dp, ctypes.c_double, ctypes.c_int32,
                                        ctypes.POINTER(ctypes.c_int32), dp]),
        "lbm_macrovar": (ctypes.c_int, [ctx, dp, dp, dp, dp]),
        "lbm_strain": (ctypes.c_int, [ctx, dp, dp]),
        "lbm_mlp_create": (ctypes.c_int, [ctypes.POINTER(ctx), ctypes.c_uint64, ctypes.c_int32]),
        "lbm_mlp_destroy": (ctypes.c_int, [ctx]),
        "lbm_mlp_get": (ctypes.c_int, [ctx, fp, fp]),
        "lbm_mlp_set": (ctypes.c_int, [ctx, fp, fp]),
        "lbm_mlp_set_data": (ctypes.c_int, [ctx, fp, fp, ctypes.c_int64, ctypes.c_int32]),
        "lbm_mlp_train": (ctypes.c_int, [ctx, ctypes.c_int32, ctypes.c_int32, ctypes.c_float, ctypes.c_int32, fp]),
        "lbm_mlp_gradient": (ctypes.c_int, [ctx, ctypes.c_int32, ctypes.POINTER(ctypes.c_double), fp]),
        "lbm_mlp_predict": (ctypes.c_int, [ctx, fp, ctypes.c_int64, fp]),
        "lbm_les_set": (ctypes.c_int, [ctx, fp, fp, ctypes.c_double, ctypes.c_double]),
        "lbm_les_wall_damping": (ctypes.c_int, [ctx, ctypes.c_double]),
        "lbm_les_nut": (ctypes.c_int, [ctx, dp]),
        "lbm_les_features": (ctypes.c_int, [ctx, ctypes.c_double, ctypes.c_double, fp]),
        "lbm_les_training_data": (ctypes.c_int, [ctx, ctypes.c_int32, ctypes.c_double, ctypes.c_double, fp, fp, dp]),
        "lbm_diag": (ctypes.c_int, [ctx, ctypes.POINTER(LBMStats)]),
        "lbm_profiles": (ctypes.c_int, [ctx, dp]),
        "lbm_profiles_noalloc": (ctypes.c_int, [ctx, dp]),
        "lbm_avedensity": (ctypes.c_int, [ctx, dp]),
        "lbm_save_flow": (ctypes.c_int, [ctx, ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
        "lbm_load_flow": (ctypes.c_int, [ctx, ctypes.c_char_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_int32)]),
        "lbm_timing_enable": (ctypes.c_int, [ctx, ctypes.c_int32]),
        "lbm_timing_get": (ctypes.c_int, [ctx, dp, dp, dp, ctypes.POINTER(ctypes.c_int64),
                                          ctypes.POINTER(ctypes.c_int64)]),
        "lbm_particle_params_init": (ctypes.c_int, [ctypes.POINTER(LBMParticleParams), ctypes.c_int32,
                                                    ctypes.c_double, ctypes.c_double]),
        "lbm_particles_place": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                               ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_uint64,
                                               dp]),
        "lbm_particles_set": (ctypes.c_int, [ctx, ctypes.POINTER(LBMParticleParams), dp, dp, dp]),
        "lbm_particles_get": (ctypes.c_int, [ctx, dp, dp, dp, dp, dp]),
        "lbm_particles_get_history": (ctypes.c_int, [ctx, dp, dp]),
        "lbm_particles_set_history": (ctypes.c_int, [ctx, dp, dp]),
        "lbm_save_part": (ctypes.c_int, [ctx, ctypes.c_char_p]),
        "lbm_dissipation": (ctypes.c_int, [ctx, dp]),
        "lbm_load_part": (ctypes.c_int, [ctx, ctypes.c_char_p, ctypes.POINTER(LBMParticleParams)]),
        "lbm_particle_counts": (ctypes.c_int, [ctx, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64),
                                               ctypes.POINTER(ctypes.c_int64)]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def _check(lib, rc: int, where: str) -> None:
    if rc != 0:
        detail = lib.lbm_last_error().decode() or lib.lbm_strerror(rc).decode()
        raise LBMError(rc, where, detail)


def _dptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _fptr(a: np.ndarray | None):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


MLP_IN, MLP_PARAMS, MLP_NORM = 7, 1345, 14
MLP_FP32 = 1


class ClosureNet:
    """The learned LES closure's eddy-viscosity network (``lbm_mlp_*``):
    7 features -> 32 -> 32 -> nu_t / nu, trained on the GPU."""

    def __init__(self, seed: int = 0, device: int = 0):
        self.lib = load_library()
        self._m = ctypes.c_void_p()
        _check(self.lib, self.lib.lbm_mlp_create(ctypes.byref(self._m), seed, device), "lbm_mlp_create")

    def close(self) -> None:
        if self._m:
            self.lib.lbm_mlp_destroy(self._m)
            self._m = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _call(self, name, *args):
        _check(self.lib, getattr(self.lib, name)(self._m, *args), name)

    def get(self) -> tuple[np.ndarray, np.ndarray]:
        p = np.empty(MLP_PARAMS, dtype=np.float32)
        n = np.empty(MLP_NORM, dtype=np.float32)
        self._call("lbm_mlp_get", _fptr(p), _fptr(n))
        return p, n

    def set(self, params=None, norm=None) -> None:
        p = None if params is None else np.ascontiguousarray(params, dtype=np.float32).reshape(MLP_PARAMS)
        n = None if norm is None else np.ascontiguousarray(norm, dtype=np.float32).reshape(MLP_NORM)
        self._call("lbm_mlp_set", _fptr(p), _fptr(n))

    def set_data(self, X, y, set_norm: bool = True) -> None:
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, MLP_IN)
        y = np.ascontiguousarray(y, dtype=np.float32).reshape(-1)
        if len(X) != len(y):
            raise ValueError("X and y differ in length")
        self._data = (X, y)
        self._call("lbm_mlp_set_data", _fptr(X), _fptr(y), len(X), int(set_norm))

    def train(self, steps: int, batch: int = 65536, lr: float = 1e-3, fp32: bool = False) -> np.ndarray:
        losses = np.empty(max(steps, 1), dtype=np.float32)
        self._call("lbm_mlp_train", steps, batch, lr, MLP_FP32 if fp32 else 0, _fptr(losses))
        return losses[:steps]

    def gradient(self, fp32: bool = False) -> tuple[float, np.ndarray]:
        loss = ctypes.c_double()
        g = np.empty(MLP_PARAMS, dtype=np.float32)
        self._call("lbm_mlp_gradient", MLP_FP32 if fp32 else 0, ctypes.byref(loss), _fptr(g))
        return loss.value, g

    def predict(self, X) -> np.ndarray:
        X = np.ascontiguousarray(X, dtype=np.float32).reshape(-1, MLP_IN)
        out = np.empty(len(X), dtype=np.float32)
        self._call("lbm_mlp_predict", _fptr(X), len(X), _fptr(out))
        return out


# --------------------------------------------------------------------------
# run constants (para.f90)
# --------------------------------------------------------------------------
@dataclass
class RunParams:
    """The scalars para.f90 sets for the channel (para.f90:59-141)."""

    nx: int              # wall-normal nodes (walls at x = 1/2 and nx + 1/2)
    ny: int              # streamwise nodes (periodic)
    nz: int              # spanwise nodes (periodic)
    visc: float
    force_y: float       # streamwise body force (force_in_y * force_mag)
    mrt_type: int = MRT_STABLE
    ustar: float = 0.0
    precision: int = PREC_FP64
    fp16_scale: float = 32768.0
    device: int = 0
    flags: int = 0
    s16: float | None = None  # rate of the third-order odd moments, overriding the MRT type's
    extra: dict = field(default_factory=dict)

    def to_c(self) -> LBMParams:
        p = LBMParams()
        lib = load_library()
        _check(lib, lib.lbm_params_init(ctypes.byref(p), self.nx, self.ny, self.nz, self.mrt_type,
                                        self.visc, self.force_y, self.precision), "lbm_params_init")
        p.fp16_scale = self.fp16_scale
        p.device = self.device
        p.flags = self.flags
        if self.s16 is not None:
            p.s16 = self.s16
        return p

    def rates(self) -> dict:
        """MRT rates and equilibrium coefficients (para.f90:106-141), computed in Python."""
        tau = 3.0 * self.visc + 0.5
        s9 = 1.0 / tau
        if self.mrt_type == MRT_STABLE:
            r = dict(s1=1.5, s2=1.4, s4=1.2, s10=1.4, s16=1.98, omegepsl=0.0, omegepslj=-475.0 / 63.0, omegxx=0.0)
        elif self.mrt_type == MRT_LBGK:
            r = dict(s1=s9, s2=s9, s4=s9, s10=s9, s16=s9, omegepsl=3.0, omegepslj=-11.0 / 2.0, omegxx=-0.5)
        elif self.mrt_type == MRT_LOWDISS:
            r = dict(s1=1.8, s2=1.8, s4=s9, s10=1.8, s16=1.8, omegepsl=3.0, omegepslj=-11.0 / 2.0, omegxx=-0.5)
        else:
            raise ValueError("mrt_type must be 1, 2 or 3")
        r.update(s9=s9, s13=s9)
        if self.s16 is not None:
            r["s16"] = self.s16
        return r


def para(nx: int, ny: int, nz: int, laminar: bool = True, **kw) -> RunParams:
    """Constants of para.f90:59-88 for an nx (wall-normal) x ny x nz lattice.

    laminar=True  -> Rstar=20, ustar=0.05 (centreline), visc = 2 ustar nx / Rstar,
                     force = 8 visc ustar / nx^2, MRTtype 2 (LBGK)
    laminar=False -> visc=0.0036, Rstar=180, ustar = 2 Rstar visc / nx,
                     force = 2 rho0 ustar^2 / nx, MRTtype 1
    """
    if laminar:
        rstar, ustar = 20.0, 0.05
        visc = 2.0 * ustar * nx / rstar
        force = 8.0 * visc * ustar / nx**2
        mrt = MRT_LBGK
    else:
        visc, rstar = 0.0036, 180.0
        ustar = 2.0 * rstar * visc / nx
        force = 2.0 * 1.0 * ustar * ustar / nx
        mrt = MRT_STABLE
    kw.setdefault("mrt_type", mrt)
    return RunParams(nx=nx, ny=ny, nz=nz, visc=visc, force_y=force, ustar=ustar, **kw)


@dataclass(frozen=True)
class ChannelConfig:
    """A channel workload in the benchmark's axes (x streamwise, y spanwise,
    z wall-normal) with its reference-axis lattice (nx wall-normal, ny
    streamwise, nz spanwise)."""

    name: str
    stream: int
    span: int
    wall: int
    visc: float
    ustar: float
    h: float
    steps: int
    precision: str = "fp64"
    uc: float = 0.05
    amp: float = 0.05
    seed: int = 20240611
    spheres: int = 0
    radius: float = 0.0
    # rate of the third-order odd moments (m_x, m_y, m_z) when it should
    # differ from the MRT type's; None keeps MRTtype 1's 1.98 (para.f90)
    s16: float | None = None

    @property
    def force(self) -> float:
        return self.ustar**2 / self.h          # gx = u*^2 / h

    @property
    def nodes(self) -> int:
        return self.stream * self.span * self.wall

    def params(self, precision: str | None = None, **kw) -> RunParams:
        prec = PRECISIONS[precision or self.precision]
        kw.setdefault("s16", self.s16)
        return RunParams(nx=self.wall, ny=self.stream, nz=self.span, visc=self.visc, force_y=self.force,
                         mrt_type=MRT_STABLE, ustar=self.ustar, precision=prec, **kw)


CHANNEL_CONFIGS = {
    # plain turbulent channel, Re_tau ~ 93
    "channel-128x64x64": ChannelConfig("channel-128x64x64", 128, 64, 64, visc=0.0012, ustar=0.0035, h=32, steps=2000),
    # particle-laden channel, Re_tau ~ 181 (fluid part)
    "spheres-256x128x128": ChannelConfig("spheres-256x128x128", 256, 128, 128, visc=0.0012, ustar=0.0034, h=64,
                        steps=5000, spheres=256, radius=4.0),
    # precision sweep, Re_tau ~ 181
    "spheres-512x256x256": ChannelConfig("spheres-512x256x256", 512, 256, 256, visc=0.0024, ustar=0.0034, h=128,
                        steps=20000, spheres=2048, radius=8.0),
    # large channel, FP32 compute / FP16 storage, Re_tau ~ 363
    "spheres-1024x512x512": ChannelConfig("spheres-1024x512x512", 1024, 512, 512, visc=0.0024, ustar=0.0034, h=256,
                        steps=2000, precision="fp16", spheres=16384, radius=8.0),
}


# --------------------------------------------------------------------------
# device lattice
# --------------------------------------------------------------------------
class Lattice:
    """Device-resident D3Q19 channel state (one GPU, one stream)."""

    def __init__(self, params: RunParams | LBMParams, lib: ctypes.CDLL | None = None):
        self.lib = lib if lib is not None else load_library()
        self.cparams = params.to_c() if isinstance(params, RunParams) else params
        self.nx, self.ny, self.nz = self.cparams.nx, self.cparams.ny, self.cparams.nz
        self._ctx = ctypes.c_void_p()
        _check(self.lib, self.lib.lbm_create(ctypes.byref(self.cparams), ctypes.byref(self._ctx)), "lbm_create")

    # lifetime ---------------------------------------------------------------
    def close(self) -> None:
        if self._ctx:
            self.lib.lbm_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # helpers ----------------------------------------------------------------
    @property
    def shape(self) -> tuple[int, int, int]:
        return (self.nx, self.ny, self.nz)

    @property
    def nodes(self) -> int:
        return self.nx * self.ny * self.nz

    def _field(self, a: np.ndarray, name: str) -> np.ndarray:
        a = np.asarray(a, dtype=np.float64)
        if a.size != self.nodes:
            raise ValueError(f"{name} must have {self.nodes} values (nx*ny*nz)")
        return np.asfortranarray(a.reshape(self.shape, order="F"))

    def _call(self, name: str, *args) -> None:
        _check(self.lib, getattr(self.lib, name)(self._ctx, *args), name)

    # reference interface ------------------------------------------------------
    def upload_f(self, f: np.ndarray) -> None:
        f = np.asarray(f, dtype=np.float64)
        if f.size != 19 * self.nodes:
            raise ValueError("f must have 19*nx*ny*nz values")
        f = np.asfortranarray(f.reshape((19,) + self.shape, order="F"))
        self._call("lbm_upload_f", _dptr(f))

    def download_f(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty((19,) + self.shape, dtype=np.float64, order="F")
        self._call("lbm_download_f", _dptr(out))
        return out

    def initpop(self, ux, uy, uz) -> None:
        a, b, c = (self._field(v, n) for v, n in ((ux, "ux"), (uy, "uy"), (uz, "uz")))
        self._call("lbm_initpop", _dptr(a), _dptr(b), _dptr(c))

    def init_channel(self, uc: float, amp: float, seed: int) -> None:
        self._call("lbm_init_channel", ctypes.c_double(uc), ctypes.c_double(amp), ctypes.c_uint64(seed))

    def init_loglaw(self, ustar: float, ystar: float, a9: float = 0.0) -> None:
        """initvel's turbulent start (law-of-the-wall profile, initial.f90:101-147)
        + initpop on the device; ystar = visc/ustar, a9 the perturbation
        amplitude A9 (0 as the reference ships it)."""
        self._call("lbm_init_loglaw", ctypes.c_double(ustar), ctypes.c_double(ystar), ctypes.c_double(a9))

    def step(self, n: int = 1) -> None:
        self._call("lbm_step", n)

    def step_async(self, n: int = 1) -> None:
        self._call("lbm_step_async", n)

    def synchronize(self) -> None:
        self._call("lbm_synchronize")

    def stream(self) -> int:
        s = ctypes.c_void_p()
        self._call("lbm_stream", ctypes.byref(s))
        return s.value or 0

    def step_count(self) -> int:
        n = ctypes.c_int64()
        self._call("lbm_step_count", ctypes.byref(n))
        return n.value

    def step_launches(self) -> int:
        """Kernels launched by the steps of this context so far."""
        n = ctypes.c_int64()
        self._call("lbm_step_launches", ctypes.byref(n))
        return n.value

    def set_step_count(self, n: int) -> None:
        self._call("lbm_set_step_count", n)

    def device_bytes(self) -> int:
        n = ctypes.c_size_t()
        self._call("lbm_device_bytes", ctypes.byref(n))
        return n.value

    def prerelax(self, ux=None, uy=None, uz=None, eps: float = 1e-5, maxit: int = 15000) -> tuple[int, float]:
        """main.f90:69-90 with the velocity frozen at (ux, uy, uz), or, all
        None, at the velocity of the current populations (device only)."""
        if ux is None and uy is None and uz is None:
            a = b = c = None
        else:
            a, b, c = (self._field(v, n) for v, n in ((ux, "ux"), (uy, "uy"), (uz, "uz")))
        it = ctypes.c_int32()
        err = ctypes.c_double()
        self._call("lbm_prerelax", _dptr(a), _dptr(b), _dptr(c), eps, maxit, ctypes.byref(it), ctypes.byref(err))
        return it.value, err.value

    def macrovar(self) -> tuple[np.ndarray, np.ndarray, np.ndarray, np.ndarray]:
        outs = [np.empty(self.shape, dtype=np.float64, order="F") for _ in range(4)]
        self._call("lbm_macrovar", *map(_dptr, outs))
        return tuple(outs)

    def les_set(self, params=None, norm=None, ustar: float = 0.0, h: float = 0.0) -> None:
        """Fuse the closure network into the collision (None: plain MRT)."""
        if params is None:
            self._call("lbm_les_set", None, None, 0.0, 0.0)
            return
        p = np.ascontiguousarray(params, dtype=np.float32).reshape(MLP_PARAMS)
        n = np.ascontiguousarray(norm, dtype=np.float32).reshape(MLP_NORM)
        self._les = (p, n)
        self._call("lbm_les_set", _fptr(p), _fptr(n), ustar, h)

    def les_wall_damping(self, aplus: float) -> None:
        """van Driest damping (1 - exp(-y+/A+))^2 of the closure's nu_t (0: off)."""
        self._call("lbm_les_wall_damping", ctypes.c_double(aplus))

    def les_training_data(self, factor: int, ustar: float, h: float):
        """(X[nc][7], y[nc], ubar[3][nxc][nyc][nzc]) of the box-filtered state."""
        nxc, nyc, nzc = (d // factor for d in self.shape)
        nc = nxc * nyc * nzc
        X = np.empty((nc, MLP_IN), dtype=np.float32)
        y = np.empty(nc, dtype=np.float32)
        ub = np.empty((3, nc), dtype=np.float64)
        self._call("lbm_les_training_data", factor, ustar, h, _fptr(X), _fptr(y), _dptr(ub))
        return X, y, ub.reshape(3, nzc, nyc, nxc).transpose(0, 3, 2, 1)

    def les_features(self, ustar: float, h: float) -> np.ndarray:
        """The closure's features per node, X[n][7], nodes in Fortran order."""
        X = np.empty((int(np.prod(self.shape)), MLP_IN), dtype=np.float32)
        self._call("lbm_les_features", ustar, h, _fptr(X))
        return X

    def les_nut(self) -> np.ndarray:
        out = np.empty(self.shape, dtype=np.float64, order="F")
        self._call("lbm_les_nut", _dptr(out))
        return out

    def strain(self) -> tuple[np.ndarray, np.ndarray]:
        """S_ij S_ij per node by the two methods of sijstat01 (moments, populations)."""
        outs = [np.empty(self.shape, dtype=np.float64, order="F") for _ in range(2)]
        self._call("lbm_strain", *map(_dptr, outs))
        return outs[0], outs[1]

    def diag(self) -> LBMStats:
        st = LBMStats()
        self._call("lbm_diag", ctypes.byref(st))
        return st

    def profiles(self) -> np.ndarray:
        """Plane sums (nx, 12) in the column order of PROFILE_NAMES."""
        out = np.empty((self.nx, PROFILE_COLS), dtype=np.float64)
        self._call("lbm_profiles", _dptr(out))
        return out

    def avedensity(self) -> float:
        m = ctypes.c_double()
        self._call("lbm_avedensity", ctypes.byref(m))
        return m.value

    # moving spheres -----------------------------------------------------------
    def set_particles(self, pos, radius: float, rho_ratio: float = 2.0, vel=None, omg=None, **overrides) -> None:
        """Attach spheres (positions (n,3), reference axes, node ix at ix-1/2)."""
        pos = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        pp = LBMParticleParams()
        _check(self.lib, self.lib.lbm_particle_params_init(ctypes.byref(pp), len(pos), radius, rho_ratio),
               "lbm_particle_params_init")
        for k, v in overrides.items():
            setattr(pp, k, v)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
        o = None if omg is None else np.ascontiguousarray(omg, dtype=np.float64).reshape(-1, 3)
        self._npart = len(pos)
        self._call("lbm_particles_set", ctypes.byref(pp), _dptr(pos), _dptr(v), _dptr(o))

    def particle_history(self) -> tuple[np.ndarray, np.ndarray]:
        """Total force and torque of the previous step (the force history)."""
        n = getattr(self, "_npart", 0)
        fp, tp = np.empty((n, 3)), np.empty((n, 3))
        self._call("lbm_particles_get_history", _dptr(fp), _dptr(tp))
        return fp, tp

    def set_particle_history(self, fprev, tprev) -> None:
        fp = np.ascontiguousarray(fprev, dtype=np.float64).reshape(-1, 3)
        tp = np.ascontiguousarray(tprev, dtype=np.float64).reshape(-1, 3)
        self._call("lbm_particles_set_history", _dptr(fp), _dptr(tp))

    def dissipation(self) -> np.ndarray:
        """dissipation_calc plane sums (saveload.f90:4644-4882): (nx, 5) =
        S_ij S_ij (moments), S_ij S_ij (f - f^eq), S_xy of both, fluid nodes."""
        out = np.empty((self.nx, DISSIPATION_COLS), dtype=np.float64)
        self._call("lbm_dissipation", _dptr(out))
        return out

    def save_part(self, path: str | Path) -> None:
        """endrunpart2D checkpoint of the spheres (savecntdpart, saveload.f90:604-647)."""
        self._call("lbm_save_part", str(path).encode())

    def load_part(self, path: str | Path, radius: float, rho_ratio: float = 2.0, **overrides) -> None:
        """Attach the spheres of an endrunpart2D checkpoint (loadcntdpart, saveload.f90:649-693)."""
        n = self.part_count(path)
        pp = LBMParticleParams()
        _check(self.lib, self.lib.lbm_particle_params_init(ctypes.byref(pp), n, radius, rho_ratio),
               "lbm_particle_params_init")
        for k, v in overrides.items():
            setattr(pp, k, v)
        self._call("lbm_load_part", str(path).encode(), ctypes.byref(pp))
        self._npart = n

    @staticmethod
    def part_count(path: str | Path) -> int:
        """nps of an endrunpart2D file (first integer of its first record)."""
        with open(path, "rb") as fh:
            head = fh.read(8)
        if len(head) < 8:
            raise ValueError(f"{path}: not a particle checkpoint")
        return int(np.frombuffer(head[4:8], dtype="<i4")[0])

    def particles(self) -> dict:
        n = getattr(self, "_npart", 0)
        out = {k: np.empty((n, 3)) for k in ("pos", "vel", "omg", "force", "torque")}
        self._call("lbm_particles_get", *(_dptr(out[k]) for k in ("pos", "vel", "omg", "force", "torque")))
        return out

    def timing_enable(self, capacity: int) -> None:
        self._call("lbm_timing_enable", capacity)

    def timing(self) -> dict:
        fe, fo, pm = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        ne, no = ctypes.c_int64(), ctypes.c_int64()
        self._call("lbm_timing_get", ctypes.byref(fe), ctypes.byref(fo), ctypes.byref(pm), ctypes.byref(ne),
                   ctypes.byref(no))
        return dict(even_ms=fe.value, odd_ms=fo.value, particle_ms=pm.value, even=ne.value, odd=no.value)

    def particle_counts(self) -> tuple[int, int, int]:
        a, b, c = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
        self._call("lbm_particle_counts", ctypes.byref(a), ctypes.byref(b), ctypes.byref(c))
        return a.value, b.value, c.value

    def save_flow(self, path: str | Path, kind: int, ints) -> None:
        arr = (ctypes.c_int32 * 3)(*list(ints) + [0] * (3 - len(ints)))
        self._call("lbm_save_flow", str(path).encode(), kind, arr)

    def load_flow(self, path: str | Path, kind: int) -> list[int]:
        arr = (ctypes.c_int32 * 3)()
        self._call("lbm_load_flow", str(path).encode(), kind, arr)
        return list(arr)[: (1 if kind == 0 else 3)]


def channel_velocity(nx: int, ny: int, nz: int, uc: float, amp: float, seed: int):
    """Host copy of the device channel initial velocity (reference layout)."""
    lib = load_library()
    out = [np.empty((nx, ny, nz), dtype=np.float64, order="F") for _ in range(3)]
    _check(lib, lib.lbm_channel_velocity(nx, ny, nz, uc, amp, ctypes.c_uint64(seed), *map(_dptr, out)),
           "lbm_channel_velocity")
    return tuple(out)


def loglaw_velocity(nx: int, ny: int, nz: int, ustar: float, ystar: float, a9: float = 0.0):
    """Host copy of the log-law initial velocity (ux, uy, uz), reference layout."""
    lib = load_library()
    out = [np.empty((nx, ny, nz), dtype=np.float64, order="F") for _ in range(3)]
    _check(lib, lib.lbm_loglaw_velocity(nx, ny, nz, ustar, ystar, a9, *map(_dptr, out)), "lbm_loglaw_velocity")
    return tuple(out)


def place_spheres(nx: int, ny: int, nz: int, npart: int, radius: float, gap: float = 2.0,
                  wall_gap: float = 1.0, seed: int = 12345) -> np.ndarray:
    """Seeded non-overlapping sphere centres (reference axes), shape (npart, 3)."""
    lib = load_library()
    pos = np.empty((npart, 3), dtype=np.float64)
    _check(lib, lib.lbm_particles_place(nx, ny, nz, npart, radius, gap, wall_gap, ctypes.c_uint64(seed),
                                        _dptr(pos)), "lbm_particles_place")
    return pos


def statistics(prof: np.ndarray, ustar: float) -> dict:
    """statistc2 normalisation (saveload.f90:1442-1462) of plane sums:
    means by u*, variances and stresses by u*^2, pressure <rho>/u*^2."""
    n = prof[:, 11]
    mean = prof[:, 0:3] / n[:, None] / ustar
    sq = prof[:, 6:9] / n[:, None] / ustar**2 - mean**2
    st = prof[:, 3:6] / n[:, None] / ustar**2
    stress = np.stack([st[:, 0] - mean[:, 0] * mean[:, 2],     # xz
                       st[:, 1] - mean[:, 0] * mean[:, 1],     # xy (wall-normal x streamwise)
                       st[:, 2] - mean[:, 1] * mean[:, 2]], 1)  # yz
    pr = prof[:, 9] / n / ustar**2
    prsq = prof[:, 10] / n / ustar**4 - pr * pr
    return dict(mean=mean, sq=sq, stress=stress, pressure=pr, pressure_sq=prsq, volf_fluid=n / n.max())
