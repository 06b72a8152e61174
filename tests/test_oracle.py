"""The oracle (oracle/physim_oracle.c) against the reference's own tests and
analytic known answers.  CPU only."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np
import pytest

GOLDEN = Path(__file__).resolve().parent / "golden"


def _entity(x, y, z, m):
    from physim_gb300.entity import entity_new
    return entity_new(x, y, z, m)


def _bodies(spec):
    from physim_gb300.entity import entities
    if isinstance(spec, list):
        return [_entity(b["x"], b["y"], b["z"], b["mass"]) for b in spec]
    rng = np.random.Generator(np.random.PCG64(spec["seed"]))
    n = spec["n"]
    if spec["gen"] == "cluster":  # (random::<f64>() - 0.5) * scale per axis
        xyz = (rng.random((n, 3)) - 0.5) * spec["scale"]
        return [_entity(*p, 1.0) for p in xyz]
    # Entity::random (physim-core/src/lib.rs:115-128): x,y in [-1,1), z in [0,1)
    s = entities(n)
    s["x"] = rng.uniform(-1.0, 1.0, n)
    s["y"] = rng.uniform(-1.0, 1.0, n)
    s["z"] = rng.uniform(0.0, 1.0, n)
    s["mass"] = 0.005
    s["radius"] = 0.02
    return list(s)


def _build(oracle_mod, kat, bodies):
    t = oracle_mod.Tree(kat["nchild"], kat["centre"], kat["extent"])
    for b in bodies:
        assert t.push(b) == 0
    return t


TREE_KATS = json.loads((GOLDEN / "tree_kats.json").read_text())


@pytest.mark.parametrize("kat", TREE_KATS, ids=[f"{k['tree']}-{k['name']}" for k in TREE_KATS])
def test_reference_tree_kats(oracle_mod, kat):
    """astro/src/octree.rs:218-519 and astro/src/quadtree.rs:197-492, as data."""
    bodies = _bodies(kat["bodies"])
    t = _build(oracle_mod, kat, bodies)
    labelled = {}
    for q in kat["queries"]:
        n = t.leaves(q["loc"], q["theta"])
        if "eq" in q:
            assert n == q["eq"], (kat["name"], q)
        if "gt" in q:
            assert n > q["gt"], (kat["name"], q)
        if "label" in q:
            labelled[q["label"]] = n
        if q.get("same_as_rebuild"):
            t2 = _build(oracle_mod, kat, _bodies(kat["bodies"]))
            assert t2.leaves(q["loc"], q["theta"]) == n
    if labelled:
        assert labelled["loose"] >= labelled["medium"] >= labelled["strict"]


def test_entity_layout(oracle_mod):
    from physim_gb300.entity import ACCELERATION, ENTITY
    lib = oracle_mod.load()
    assert lib.oracle_sizeof_entity() == ENTITY.itemsize == 80
    assert lib.oracle_sizeof_acceleration() == ACCELERATION.itemsize == 24


LAW = json.loads((GOLDEN / "law_kats.json").read_text())


@pytest.mark.parametrize("case", LAW["pairs"])
def test_law_known_answers(oracle_mod, case):
    """astro/src/lib.rs:84-113 on separations with whole-number r."""
    a = _entity(*case["a"], case["ma"])
    b = _entity(*case["b"], case["mb"])
    f = oracle_mod.law(a, b, case["e"])
    np.testing.assert_allclose(f, case["force"], rtol=4e-16, atol=1e-300)


def test_direct_sum_known_answer(oracle_mod):
    from physim_gb300.entity import accelerations, entities
    d = LAW["direct3"]
    s = entities(3)
    for i, (x, y, z, m) in enumerate(d["bodies"]):
        s[i]["x"], s[i]["y"], s[i]["z"], s[i]["mass"] = x, y, z, m
    acc = oracle_mod.simple_astro(s, d["e"], accelerations(3))
    np.testing.assert_allclose([acc[0]["x"], acc[0]["y"], acc[0]["z"]], d["acc0"], rtol=1e-15,
                               atol=1e-300)


def test_equal_positions_are_skipped(oracle_mod):
    """transformers.rs:230: pairs at exactly the same centre contribute nothing."""
    from physim_gb300.entity import accelerations, entities
    s = entities(3)
    s["x"] = [0.0, 0.0, 1.0]
    s["mass"] = [1.0, 2.0, 3.0]
    acc = oracle_mod.simple_astro(s, 0.5, accelerations(3))
    # body 0 sees only body 2: (1,0,0)/1 * 1*3/(1+0.5) / 1
    assert acc[0]["x"] == pytest.approx(2.0, rel=1e-15)
    assert acc[0]["y"] == 0.0 and acc[0]["z"] == 0.0


def test_massless_body_gets_nan(oracle_mod):
    """F/m_i with m_i = 0 is 0/0 in the reference (transformers.rs:236-240)."""
    from physim_gb300.entity import accelerations, entities
    s = entities(2)
    s["x"] = [0.0, 1.0]
    s["mass"] = [0.0, 1.0]
    acc = oracle_mod.simple_astro(s, 0.1, accelerations(2))
    assert np.isnan(acc[0]["x"]) and np.isnan(acc[0]["y"])
    assert np.isfinite(acc[1]["x"])


def test_fixed_bodies_untouched(oracle_mod):
    from physim_gb300.entity import accelerations, entities
    s = entities(2)
    s["x"] = [0.0, 1.0]
    s["mass"] = 1.0
    s["fixed"][0] = 1
    acc = accelerations(2)
    acc["x"] = [-0.0, 5.0]
    oracle_mod.simple_astro(s, 0.1, acc)
    assert np.signbit(acc[0]["x"])  # untouched, still -0.0
    assert acc[1]["x"] != 5.0


def test_verlet_known_steps(oracle_mod):
    """verlet.rs:24-82 by hand: Taylor first step, then position verlet."""
    from physim_gb300.entity import accelerations, entities
    s = entities(1)
    s["x"], s["vx"], s["mass"] = 1.0, 2.0, 1.0
    a = accelerations(1)
    a["x"] = 4.0
    v = oracle_mod.Verlet()
    dt = 0.5
    s1 = v.step(s, a, dt)
    assert s1["x"][0] == 1.0 + 2.0 * 0.5 + 0.5 * 4.0 * 0.25
    assert s1["vx"][0] == 2.0 + 4.0 * 0.5
    s2 = v.step(s1, a, dt)
    x2 = 2.0 * s1["x"][0] - 1.0 + 4.0 * 0.25
    assert s2["x"][0] == x2
    assert s2["vx"][0] == (x2 - s1["x"][0]) / dt
    # a different length restarts with the Taylor step (verlet.rs:102)
    s3 = v.step(np.concatenate([s2, s2]), np.concatenate([a, a]), dt)
    assert s3["vx"][0] == s2["vx"][0] + 4.0 * 0.5


def test_euler_known_step(oracle_mod):
    """euler.rs:29-37 by hand; fixed bodies drift (euler ignores `fixed`)."""
    from physim_gb300.entity import accelerations, entities
    s = entities(2)
    s["x"], s["vx"], s["mass"] = 1.0, 2.0, 1.0
    s["fixed"][1] = 1
    a = accelerations(2)
    a["x"] = 4.0
    s1 = oracle_mod.euler_step(s, a, 0.5)
    assert np.all(s1["x"] == 1.0 + 2.0 * 0.5 + 0.5 * 4.0 * 0.25)
    assert np.all(s1["vx"] == 2.0 + 4.0 * 0.5)
    assert s1["fixed"][1] == 1


def _rk4_numpy(s, acc_of, dt):
    """rk4.rs:24-178 restated with numpy arrays (independent of the C oracle)."""
    x = np.stack([s["x"], s["y"], s["z"]], 1)
    v = np.stack([s["vx"], s["vy"], s["vz"]], 1)
    ks = []
    qx, qv = x, v
    for c in (0.5, 0.5, 1.0, None):
        a = acc_of(qx)
        kx, kv = dt * qv, dt * a
        ks.append((kx, kv))
        if c is not None:
            qx, qv = (x + 0.5 * kx, v + 0.5 * kv) if c == 0.5 else (x + kx, v + kv)
    sx = ks[0][0] + 2.0 * ks[1][0] + 2.0 * ks[2][0] + ks[3][0]
    sv = ks[0][1] + 2.0 * ks[1][1] + 2.0 * ks[2][1] + ks[3][1]
    nx, nv = x + sx / 6.0, v + sv / 6.0
    fixed = s["fixed"].astype(bool)
    nx[fixed], nv[fixed] = x[fixed], 0.0
    return nx, nv


def test_rk4_matches_numpy_restatement(oracle_mod):
    """The C rk4 step equals an independent numpy restatement bit for bit
    (harmonic force a = -k x, evaluated on the stage states), including a
    fixed body (rk4.rs:165-171: position kept, velocity zeroed)."""
    from physim_gb300 import ics
    s = ics.cube_with_stars(64, seed=9)
    s["fixed"][2] = 1
    k = 3.7

    def acc_fn(state, acc):
        acc["x"] += -k * state["x"]
        acc["y"] += -k * state["y"]
        acc["z"] += -k * state["z"]

    got = oracle_mod.rk4_step(s, acc_fn, 1e-2)
    nx, nv = _rk4_numpy(s, lambda q: -k * q, 1e-2)
    assert np.array_equal(np.stack([got["x"], got["y"], got["z"]], 1), nx)
    assert np.array_equal(np.stack([got["vx"], got["vy"], got["vz"]], 1), nv)
    assert got["vx"][2] == 0.0 and got["x"][2] == s["x"][2]


def test_rk4_harmonic_accuracy(oracle_mod):
    """One-body harmonic oscillator: rk4's global error is O(dt^4)."""
    from physim_gb300.entity import entities
    s = entities(1)
    s["x"], s["mass"] = 1.0, 1.0

    def acc_fn(state, acc):
        acc["x"] += -state["x"]

    errs = []
    for dt in (0.1, 0.05):
        q = s.copy()
        for _ in range(int(round(1.0 / dt))):
            q = oracle_mod.rk4_step(q, acc_fn, dt)
        errs.append(abs(q["x"][0] - np.cos(1.0)))
    assert errs[1] < errs[0] / 12  # 2^4 = 16 in the limit


def test_pipeline_integrators(oracle_mod):
    """The pipeline loop with each integrator equals stepping by hand (field
    by field: the Entity padding bytes are not state)."""
    from physim_gb300 import ics

    def same(a, b):
        return all(a[f].tobytes() == b[f].tobytes() for f in a.dtype.names)

    s = ics.cube_with_stars(100, seed=4, stars=ics.STARS_2)
    e, dt = 0.01, 1e-5
    want = s
    for _ in range(3):
        want = oracle_mod.rk4_step(want, lambda st, ac: oracle_mod.simple_astro(st, e, ac), dt)
    got = oracle_mod.run_pipeline(s, "simple_astro", 3, dt, e, integrator="rk4")
    assert same(got, want)
    want = s
    for _ in range(3):
        want = oracle_mod.euler_step(want, oracle_mod.simple_astro(want, e), dt)
    got = oracle_mod.run_pipeline(s, "simple_astro", 3, dt, e, integrator="euler")
    assert same(got, want)


def test_barnes_hut_theta_negative_is_direct_sum(oracle_mod):
    """theta < 0 opens every cell, so astro2/astro equal simple_astro up to
    summation order."""
    from physim_gb300 import ics
    s = ics.cube_with_stars(300, seed=3, stars=ics.STARS_2)
    d = oracle_mod.simple_astro(s, 0.01)
    for nchild in (8, 4):
        b = oracle_mod.barnes_hut(s, -1.0, 0.01, nchild=nchild)
        for c in "xyz":
            np.testing.assert_allclose(b[c], d[c], rtol=1e-9, atol=1e-9)


def test_quadtree_panics_on_equal_xy(oracle_mod):
    """quadtree.rs:59-62: bodies with equal x,y but different z never separate."""
    t = oracle_mod.Tree(4, (0, 0, 0), 1.0)
    assert t.push(_entity(0.1, 0.1, 0.0, 1.0)) == 0
    assert t.push(_entity(0.1, 0.1, 0.5, 1.0)) == 1


def test_oracle_regression_fixtures(oracle_mod):
    """The oracle reproduces the committed outputs bit for bit."""
    from physim_gb300.entity import ACCELERATION, ENTITY
    f = np.load(GOLDEN / "oracle_fixtures.npz")
    st = f["state"].view(ENTITY)
    acc = lambda k: f[k].view(ACCELERATION)  # noqa: E731
    got = oracle_mod.simple_astro(st, 0.01)
    assert got.tobytes() == acc("acc_direct").tobytes()
    assert oracle_mod.barnes_hut(st, 0.5, 0.01, 8).tobytes() == acc("acc_octree").tobytes()
    assert oracle_mod.barnes_hut(st, 0.7, 0.01, 4).tobytes() == acc("acc_quadtree").tobytes()
    t1 = oracle_mod.run_pipeline(st, "simple_astro", 3, 1e-5, 0.01)
    t2 = oracle_mod.run_pipeline(st, "astro2", 3, 1e-5, 0.01, theta=1.0)
    for got_s, key in ((t1, "traj_direct"), (t2, "traj_astro2")):
        want = f[key].view(ENTITY)
        for field in ENTITY.names:  # field by field: struct padding is not data
            assert got_s[field].tobytes() == want[field].tobytes(), (key, field)


def test_parallel_sample_matches_serial(oracle_mod):
    from physim_gb300 import ics
    s = ics.cube_with_stars(500, seed=9, stars=ics.STARS_2)
    full = oracle_mod.simple_astro(s, 0.02)
    idx = np.array([0, 17, 250, 499, 500, 501])
    samp = oracle_mod.simple_astro_sample(s, 0.02, idx, threads=4)
    assert samp.tobytes() == full[idx].tobytes()
    bh_full = oracle_mod.barnes_hut(s, 0.8, 0.02, 8, threads=1)
    bh_samp = oracle_mod.barnes_hut(s, 0.8, 0.02, 8, idx=idx, threads=3)
    assert bh_samp.tobytes() == bh_full[idx].tobytes()
