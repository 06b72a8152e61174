"""The allocation-free entry point, physim_gpu_simple_astro_accumulate_static.

It exists for callers that cannot allocate device memory themselves (code
inside another framework's memory pool, a real-time loop that must not call
cudaMalloc): they hand over device-accessible arrays and the entry point
keeps its scratch in a fixed static device array.  This file is collected
last on purpose, so a run that stops at the first failure has already run
every other test.  The tests allocate their own device buffers (with torch);
the entry point allocates nothing, which is checked too: after a first call
(which may load the library's kernels), two more calls leave the device's
free memory and torch's reserved memory unchanged.  Results must match the
plugin's simple_astro_transform and the f64 oracle (astro/src/
transformers.rs:219-244) within the suite's tolerance (relative 1e-5 per
body; fixed bodies untouched; massless bodies NaN like the reference), on
two calls in a row, up to the 65,536-body limit.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-5
MAX_BODIES = 65536


def _vec(acc):
    return np.stack([acc["x"], acc["y"], acc["z"]], axis=1)


def _close(got, want, fixed):
    g, w = _vec(got), _vec(want)
    assert g[fixed].tobytes() == w[fixed].tobytes()
    nan = np.isnan(w).any(axis=1)
    assert np.array_equal(np.isnan(g).any(axis=1), nan)
    live = ~fixed & ~nan
    err = np.linalg.norm(g - w, axis=1) / np.maximum(np.linalg.norm(w, axis=1), 1e-300)
    assert err[live].max() < RTOL, err[live].max()


def _entry():
    import physim_gb300 as pg
    fn = pg.lib.physim_gpu_simple_astro_accumulate_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_double, C.c_void_p, C.c_void_p]
    return fn


def _state(n, seed):
    from physim_gb300 import ics
    state = ics.cube_with_stars(n - 2, seed=seed, stars=ics.STARS_2)
    state["fixed"][[5, 77]] = 1
    state["mass"][[11, n // 2]] = 0.0  # massless: the reference's F / m_i = NaN
    return state


def _run_device(fn, state, acc0, e, calls):
    """`calls` calls in a row on caller-owned device arrays; the
    accelerations after each call."""
    import torch

    import physim_gb300 as pg
    d_state = torch.from_numpy(state.view(np.uint8).copy()).cuda()
    d_acc = torch.from_numpy(acc0.view(np.uint8).copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    out = []
    for _ in range(calls):
        rc = fn(d_state.data_ptr(), len(state), e, d_acc.data_ptr(), stream)
        assert rc == 0, pg.last_error()
        torch.cuda.synchronize()
        out.append(d_acc.cpu().numpy().view(pg.ACCELERATION).copy())
    return out


def test_static_entry_matches_transform_and_oracle_twice(oracle_mod):
    import physim_gb300 as pg
    state = _state(6000, seed=91)
    n = len(state)
    acc0 = pg.accelerations(n)
    acc0["x"] = np.linspace(-2.0, 2.0, n)
    acc0["y"] = -0.0

    # the existing entry point, twice in a row, and the oracle
    ref1 = acc0.copy()
    with pg.TransformElementHandler("simple_astro", {"e": 0.01}) as el:
        el.transform(state, ref1)
        ref2 = ref1.copy()
        el.transform(state, ref2)
    orc1 = oracle_mod.simple_astro(state, 0.01, acc0.copy())
    orc2 = oracle_mod.simple_astro(state, 0.01, orc1.copy())

    fixed = state["fixed"].astype(bool)
    got = _run_device(_entry(), state, acc0, 0.01, 2)
    for g, want, orc in zip(got, (ref1, ref2), (orc1, orc2)):
        _close(g, want, fixed)
        _close(g, orc, fixed)


def test_static_entry_at_the_size_limit(oracle_mod):
    """65,536 bodies fill the padded body region and the partial sums; a
    negative easing is used as |e| (transformers.rs:246-256)."""
    import physim_gb300 as pg
    state = _state(MAX_BODIES, seed=92)
    acc0 = pg.accelerations(MAX_BODIES)
    with pg.TransformElementHandler("simple_astro", {"e": -0.02}) as el:
        want = acc0.copy()
        el.transform(state, want)
    fixed = state["fixed"].astype(bool)
    got = _run_device(_entry(), state, acc0, -0.02, 2)
    _close(got[0], want, fixed)
    twice = want.copy()
    for c in "xyz":
        twice[c] = np.where(fixed, want[c], 2.0 * want[c])
    _close(got[1], twice, fixed)
    idx = np.arange(0, MAX_BODIES, 257)
    orc = oracle_mod.simple_astro_sample(state, 0.02, idx)
    _close(got[0][idx], orc, fixed[idx])


def test_static_entry_allocates_nothing():
    import torch

    import physim_gb300 as pg
    state = _state(20000, seed=93)
    fn = _entry()
    d_state = torch.from_numpy(state.view(np.uint8).copy()).cuda()
    d_acc = torch.zeros(len(state) * 24, dtype=torch.uint8, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert fn(d_state.data_ptr(), len(state), 0.01, d_acc.data_ptr(), stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    reserved0 = torch.cuda.memory_reserved()
    for _ in range(2):
        assert fn(d_state.data_ptr(), len(state), 0.01, d_acc.data_ptr(), stream) == 0, \
            pg.last_error()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0 and torch.cuda.memory_reserved() == reserved0


def test_static_entry_host_arrays():
    """Pageable host arrays: used in place where the device reaches pageable
    memory (GB300 over NVLink-C2C), else rejected before any device work."""
    import physim_gb300 as pg
    state = _state(3000, seed=94)
    acc = pg.accelerations(len(state))
    fn = _entry()
    rc = fn(state.ctypes.data, len(state), 0.01, acc.ctypes.data, None)
    if pg.host_access(0) == "direct":
        assert rc == 0, pg.last_error()
        import torch
        torch.cuda.synchronize()
        want = _run_device(fn, state, pg.accelerations(len(state)), 0.01, 1)[0]
        assert _vec(acc).tobytes() == _vec(want).tobytes()
    else:
        assert rc == 1 and "pageable host memory" in pg.last_error()


def test_static_entry_rejects_oversized_state():
    import physim_gb300 as pg
    rc = _entry()(C.c_void_p(16), MAX_BODIES + 1, 0.01, C.c_void_p(16), None)
    assert rc == 1  # PHYSIM_ERR_ARGUMENT, before any device work
    assert "65536" in pg.last_error()
