"""Host arrays read and written in place by the kernels (host access DIRECT)
against the same calls with explicit copies (COPY): the transform elements and
the host-array verlet integrator must give bit-identical results either way,
for ragged sizes, fixed bodies whose accelerations must stay untouched, and
arrays that start 8 bytes off a 16-byte boundary (the kernels' narrower
copy path)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def direct():
    import physim_gb300 as pg
    pg.set_host_access("auto")
    if pg.host_access(0) != "direct":
        pytest.skip("device has no pageable host memory access")
    yield
    pg.set_host_access("auto")


def _offset_copy(a: np.ndarray, offset: int) -> np.ndarray:
    """A copy of `a` whose data starts `offset` bytes past a 16-byte boundary."""
    raw = np.zeros(a.nbytes + 32, np.uint8)
    start = (-raw.ctypes.data) % 16 + offset
    out = raw[start:start + a.nbytes].view(a.dtype)
    out[:] = a
    assert out.ctypes.data % 16 == offset
    return out


def _same_records(a, b):
    """Every field equal bit for bit (numpy's copies of structured arrays do
    not carry the records' padding bytes, so whole-record bytes can differ)."""
    assert len(a) == len(b)
    for f in a.dtype.names:
        assert a[f].tobytes() == b[f].tobytes(), f


def _state(n, seed):
    from physim_gb300 import ics
    s = ics.cube_with_stars(max(n - 2, 0), seed=seed, stars=ics.STARS_2[: min(n, 2)])
    if n > 7:
        s["fixed"][n // 5] = 1
        s["fixed"][n - 1] = 1
    return s


def _acc0(n, seed):
    import physim_gb300 as pg
    rng = np.random.default_rng(seed)
    acc = pg.accelerations(n)
    for c in "xyz":
        acc[c] = rng.normal(0, 1.0, n)
    acc["x"][:3] = [np.nan, -0.0, np.inf][: min(n, 3)]
    return acc


def _transform(name, props, state, acc0, mode, offset):
    import physim_gb300 as pg
    pg.set_host_access(mode)
    s = _offset_copy(state, offset)
    acc = _offset_copy(acc0, offset)
    with pg.TransformElementHandler(name, props) as el:
        el.transform(s, acc)
        el.transform(s, acc)  # a second call reuses the element's buffers
    _same_records(s, state)  # the state is only read
    return acc.copy()


ELEMENTS = [
    ("simple_astro", {"e": 0.01}),
    ("astro2", {"e": 0.01, "theta": 0.5, "leaf_size": 16, "traversal": "warp"}),
    ("astro2", {"e": 0.01, "theta": 0.7}),
    ("astro", {"e": 0.01, "theta": 0.5}),
]


@pytest.mark.parametrize("name,props", ELEMENTS)
@pytest.mark.parametrize("n", [1, 5, 255, 257, 3001, 40_000])
@pytest.mark.parametrize("offset", [0, 8])
def test_transform_direct_equals_copy(direct, name, props, n, offset):
    s = _state(n, seed=n + 11)
    acc0 = _acc0(n, seed=n)
    a = _transform(name, props, s, acc0, "copy", offset)
    b = _transform(name, props, s, acc0, "direct", offset)
    assert a.tobytes() == b.tobytes()
    fixed = s["fixed"].astype(bool)
    assert a[fixed].tobytes() == acc0[fixed].tobytes()


@pytest.mark.parametrize("offset", [0, 8])
def test_verlet_direct_equals_copy(direct, offset):
    import physim_gb300 as pg
    s0 = _state(5003, seed=9)
    results = {}
    for mode in ("copy", "direct"):
        pg.set_host_access(mode)
        gv = pg.GpuVerlet()
        s = s0.copy()
        out = []
        # same length (regular steps) and a length change (Taylor restart)
        for step, n in enumerate((5003, 5003, 5003, 4001, 4001)):
            s = _offset_copy(s[:n], offset)
            acc = _offset_copy(pg.accelerations(n), offset)
            r = np.random.default_rng(step)
            for c in "xyz":
                acc[c] = r.normal(0, 1e3, n)
            s = gv.integrate(s, acc, 1e-5 * (1 + step))
            out.append(s.copy())
        gv.close()
        results[mode] = out
    for a, b in zip(results["copy"], results["direct"]):
        _same_records(a, b)


def test_direct_pipeline_matches_oracle(direct, oracle_mod):
    """Two plugin pipeline steps (transform + verlet) in DIRECT mode against
    the oracle's pipeline (pipeline.rs:137-173)."""
    import physim_gb300 as pg
    from test_verlet_gpu import _trajectory_check
    pg.set_host_access("direct")
    s = _state(3000, seed=21)
    el = pg.TransformElementHandler("simple_astro", {"e": 0.01})
    gv = pg.GpuVerlet()
    cur = s.copy()
    for _ in range(2):
        acc = pg.accelerations(len(cur))
        el.transform(cur, acc)
        cur = gv.integrate(cur, acc, 1e-4)
    el.destroy()
    gv.close()
    want = oracle_mod.run_pipeline(s, "simple_astro", 2, 1e-4, 0.01)
    _trajectory_check(cur, want, s)


def test_verlet_into_reused_output(oracle_mod):
    """GpuVerlet.integrate(..., out=) writes the new state into a caller's
    array reused across steps (as physim's pipeline reuses new_state,
    pipeline.rs:104-173), identical to fresh outputs and to the oracle."""
    import physim_gb300 as pg
    s0 = _state(3001, seed=4)
    rng = np.random.default_rng(8)
    accs = []
    for _ in range(3):
        acc = pg.accelerations(len(s0))
        for c in "xyz":
            acc[c] = rng.normal(0, 1e3, len(s0))
        accs.append(acc)
    fresh, reused = pg.GpuVerlet(), pg.GpuVerlet()
    ov = oracle_mod.Verlet()
    a = b = c = s0.copy()
    buf = [np.empty_like(s0), np.empty_like(s0)]
    for k, acc in enumerate(accs):
        a = fresh.integrate(a, acc, 1e-5)
        b = reused.integrate(b, acc, 1e-5, out=buf[k % 2])
        assert b is buf[k % 2]
        c = ov.step(c, acc, 1e-5)
        _same_records(a, b)
        _same_records(a, c)
    fresh.close()
    reused.close()
    with pytest.raises(ValueError):
        pg.GpuVerlet().integrate(s0, accs[0], 1e-5, out=np.empty(5, pg.ENTITY))
