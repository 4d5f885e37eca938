"""Regenerate the golden fixtures from the FP64 oracle.

    python tests/golden/make_golden.py

The fixtures pin the oracle (the CPU tests check that it still reproduces
them bit for bit) and give the GPU tests a committed target that needs no
oracle run.  Case: a 6 x 10 x 4 channel (nx wall-normal, ny streamwise, nz
spanwise) with the MRT rates of para.f90 MRTtype 1 at visc = 0.0012, a
streamwise force, the seeded Poiseuille + noise velocity and a seeded
non-equilibrium perturbation of the populations, after 1, 2, 5 and 40 steps
of the reference's swap sweep.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1] / "oracle"))
import oracle as orc  # noqa: E402

SHAPE = (6, 10, 4)
VISC = 0.0012
FORCE = (0.0, 2.0e-5, 0.0)
SEED = 4242
STEPS = (1, 2, 5, 40)


def rates():
    s9 = 1.0 / (3 * VISC + 0.5)
    return dict(s1=1.5, s2=1.4, s4=1.2, s9=s9, s10=1.4, s13=s9, s16=1.98,
                omegepsl=0.0, omegepslj=-475.0 / 63.0, omegxx=0.0)


def initial_state():
    u = orc.channel_velocity(*SHAPE, 0.05, 0.05, SEED)
    f = orc.initpop(*u)
    rng = np.random.default_rng(SEED)
    return np.asfortranarray(f + 1e-4 * rng.standard_normal(f.shape))


def make():
    p = orc.params(rates(), FORCE)
    f0 = initial_state()
    out = {"f0": f0, "steps": np.array(STEPS), "shape": np.array(SHAPE), "visc": VISC,
           "force": np.array(FORCE)}
    for n in STEPS:
        f, rho, ux, uy, uz = orc.run(p, f0, n, mode=0)
        out[f"f{n}"] = f
        out[f"macro{n}"] = np.stack([rho, ux, uy, uz])
    return out


if __name__ == "__main__":
    np.savez_compressed(HERE / "channel_6x10x4.npz", **make())
    print("wrote", HERE / "channel_6x10x4.npz")
