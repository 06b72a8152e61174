"""The allocation-free entry point, physim_gpu_simple_astro_accumulate_static.

It exists for callers that cannot allocate device memory themselves (code
inside another framework's memory pool, a real-time loop that must not call
cudaMalloc): they hand over device-accessible arrays and the entry point
keeps its scratch in a fixed static device array.  This file is collected
last on purpose, so a run that stops at the first failure has already run
every other test.  The test allocates its own device buffers (with torch);
the entry point allocates nothing.  Its results must match the plugin's
simple_astro_transform on the same state within the suite's tolerance
(relative 1e-5 per body; fixed bodies untouched), on two calls in a row.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-5


def _vec(acc):
    return np.stack([acc["x"], acc["y"], acc["z"]], axis=1)


def _close(got, want, fixed):
    g, w = _vec(got), _vec(want)
    assert g[fixed].tobytes() == w[fixed].tobytes()
    err = np.linalg.norm(g - w, axis=1) / np.maximum(np.linalg.norm(w, axis=1), 1e-300)
    assert err[~fixed].max() < RTOL, err[~fixed].max()


def test_static_entry_matches_transform_twice():
    import torch

    import physim_gb300 as pg
    from physim_gb300 import ics
    fn = pg.lib.physim_gpu_simple_astro_accumulate_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_double, C.c_void_p, C.c_void_p]

    state = ics.cube_with_stars(6000, seed=91, stars=ics.STARS_2)
    state["fixed"][[5, 77]] = 1
    n = len(state)
    acc0 = pg.accelerations(n)
    acc0["x"] = np.linspace(-2.0, 2.0, n)
    acc0["y"] = -0.0

    # the existing entry point, twice in a row
    ref1 = acc0.copy()
    with pg.TransformElementHandler("simple_astro", {"e": 0.01}) as el:
        el.transform(state, ref1)
        ref2 = ref1.copy()
        el.transform(state, ref2)

    # buffers owned by the caller
    d_state = torch.from_numpy(state.view(np.uint8).copy()).cuda()
    d_acc = torch.from_numpy(acc0.view(np.uint8).copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    fixed = state["fixed"].astype(bool)
    for want in (ref1, ref2):
        rc = fn(d_state.data_ptr(), n, 0.01, d_acc.data_ptr(), stream)
        assert rc == 0, pg.last_error()
        torch.cuda.synchronize()
        got = d_acc.cpu().numpy().view(pg.ACCELERATION)
        _close(got, want, fixed)


def test_static_entry_rejects_oversized_state():
    import physim_gb300 as pg
    fn = pg.lib.physim_gpu_simple_astro_accumulate_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_double, C.c_void_p, C.c_void_p]
    rc = fn(C.c_void_p(16), 65537, 0.01, C.c_void_p(16), None)
    assert rc == 1  # PHYSIM_ERR_ARGUMENT, before any device work
    assert "65536" in pg.last_error()
