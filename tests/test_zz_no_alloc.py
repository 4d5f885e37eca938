"""lbm_profiles_noalloc: the profile statistics for callers that cannot
allocate device memory.

Who needs it: a statistics monitor that samples the plane-averaged profiles
while the solver owns a fixed GPU memory budget, code that runs between the
captures of a CUDA graph (where a cudaMalloc would break the capture), or an
embedding host whose memory comes from its own allocator rather than the CUDA
runtime.  lbm_profiles may allocate a reduction buffer the first time it is
called; the no-allocation variant keeps its partial sums in a fixed device
array inside the library instead.

This file is collected last on purpose, so that a run stopping at the first
failure has already run every other test.  It passes alone in a fresh process
and after the rest of the suite.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def check_close(out, ref):
    # both are FP64 sums of the same terms, only grouped differently
    scale = np.maximum(np.abs(ref).max(axis=0), 1e-300)
    assert np.all(np.abs(out - ref) <= 1e-12 * scale + 1e-10 * np.abs(ref))


@pytest.mark.parametrize("prec", ["fp64", "fp16"])
def test_noalloc_profiles_match_lbm_profiles(pkg, prec):
    lib = pkg.load_library()
    ch = pkg.CHANNEL_CONFIGS["channel-128x64x64"]
    with pkg.Lattice(ch.params(prec)) as lat:
        lat.init_channel(ch.uc, ch.amp, ch.seed)
        for steps in (7, 1):                      # swapped, then natural AA state
            lat.step(steps)
            ref = lat.profiles()
            for _ in range(2):                    # two calls in a row share the array
                out = np.full((lat.nx, pkg.PROFILE_COLS), np.nan)
                rc = lib.lbm_profiles_noalloc(lat._ctx, pkg._dptr(out))
                assert rc == 0, lib.lbm_last_error()
                assert np.isfinite(out).all()
                check_close(out, ref)
        assert ref[:, 11].sum() == lat.nodes     # every node counted once


def test_noalloc_rejects_too_many_planes(pkg):
    lib = pkg.load_library()
    run = pkg.RunParams(nx=4097, ny=8, nz=1, visc=0.01, force_y=0.0)
    with pkg.Lattice(run) as lat:
        out = np.zeros((lat.nx, pkg.PROFILE_COLS))
        rc = lib.lbm_profiles_noalloc(lat._ctx, pkg._dptr(out))
        assert rc == -1
        assert b"LBM_NOALLOC_MAX_PLANES" in lib.lbm_last_error()
        assert not out.any()
