"""The FP32 pair law over coordinate scales far from 1 (astro/src/lib.rs:84-113,
transformers.rs:219-244 for simple_astro, :122-160 for astro2, :31-69 for astro).

The pair kernels evaluate 1/sqrt(r^2 (r^2 + e)^2) in FP32; unscaled, that
argument overflows for separations above ~2.6e6 and, with e = 0, underflows
for separations below ~5e-7.  Positions enter the pair arithmetic scaled by a
power of two taken from the largest |coordinate| (PairScale in csrc/engine.h),
so these states must match the f64 oracle like unit-size ones: per-body
relative error below 1e-5 for the direct sums (both plans, the allocation of
an ensemble included) and for leaf-1 Barnes-Hut with the exact traversal
(the reference's interaction lists).

The states are jittered grids, so the f32 rounding of positions stays small
against the separations (as in a unit cube) and no two bodies come within
the reference's 1e-9 coincidence distance (octree.rs:69-80)."""
from __future__ import annotations

import numpy as np
import pytest

from test_direct_gpu import RTOL, _vec, rel_err

pytestmark = pytest.mark.gpu


def jittered_grid(m: int, spacing: float, seed: int, mass_scale: float = 1.0):
    """m^3 bodies on a grid of the given spacing centred at the origin, each
    moved by up to 0.3 spacing per axis, masses in [0.5, 1.5) * mass_scale,
    plus two bodies of 100 * mass_scale outside the grid (as the heavy stars
    of the benchmark workloads, they keep every body's net acceleration well
    away from cancelling, so relative errors per body stay meaningful)."""
    import physim_gb300 as pg
    rng = np.random.default_rng(seed)
    g = (np.arange(m) - (m - 1) / 2.0) * spacing
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    pos = pos + rng.uniform(-0.3, 0.3, pos.shape) * spacing
    half = m / 2.0 * spacing
    pos = np.concatenate([pos, [[0.7 * half, 0.7 * half, 1.6 * half],
                                [-0.7 * half, -0.7 * half, 1.6 * half]]])
    s = pg.entities(len(pos))
    s["x"], s["y"], s["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
    s["mass"] = np.concatenate([rng.uniform(0.5, 1.5, len(pos) - 2), [1e4, 1e4]]) * mass_scale
    s["radius"] = 1.0
    s["id"] = np.arange(len(pos))
    return s


# (name, grid side, spacing, e): coordinates of order 1e7 with a negligible and
# with a comparable easing, of order 1e-7 with e = 0, and an e = 0 cluster
# whose bodies are ~1e-6 apart
CASES = [("large", 12, 2e6, 0.01), ("large_e", 12, 2e6, 4e12), ("small", 12, 2e-8, 0.0),
         ("cluster_e0", 10, 1e-6, 0.0)]


def _case(name):
    for c in CASES:
        if c[0] == name:
            return c
    raise KeyError(name)


@pytest.mark.parametrize("name", [c[0] for c in CASES])
def test_direct_one_pair_plan(oracle_mod, name):
    import physim_gb300 as pg
    _, m, spacing, e = _case(name)
    s = jittered_grid(m, spacing, seed=m)
    acc = pg.accelerations(len(s))
    with pg.TransformElementHandler("simple_astro", {"e": e}) as el:
        el.transform(s, acc)
    want = oracle_mod.simple_astro(s, e)
    assert np.isfinite(_vec(acc)).all()
    err = rel_err(acc, want)
    assert err.max() < RTOL, (name, err.max())


@pytest.mark.parametrize("name", [c[0] for c in CASES])
def test_direct_each_pair_once_plan(oracle_mod, name):
    import physim_gb300 as pg
    _, m, spacing, e = _case(name)
    s = jittered_grid(m, spacing, seed=m + 1)
    with pg.Simulation(s, pg.SimConfig(gravity="simple_astro", e=e)) as sim:
        sim.set_plan(symmetric=True)
        got = sim.accelerations()
    want = oracle_mod.simple_astro(s, e)
    err = rel_err(got, want)
    assert err.max() < RTOL, (name, err.max())


def test_static_entry_point_at_large_coordinates(oracle_mod):
    import ctypes as C

    import torch

    import physim_gb300 as pg
    fn = pg.lib.physim_gpu_simple_astro_accumulate_static
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_size_t, C.c_double, C.c_void_p, C.c_void_p]
    s = jittered_grid(12, 2e6, seed=5)
    acc = pg.accelerations(len(s))
    d_state = torch.from_numpy(s.view(np.uint8).copy()).cuda()
    d_acc = torch.from_numpy(acc.view(np.uint8).copy()).cuda()
    assert fn(d_state.data_ptr(), len(s), 0.01, d_acc.data_ptr(),
              torch.cuda.current_stream().cuda_stream) == 0, pg.last_error()
    torch.cuda.synchronize()
    got = d_acc.cpu().numpy().view(pg.ACCELERATION)
    assert rel_err(got, oracle_mod.simple_astro(s, 0.01)).max() < RTOL


@pytest.mark.parametrize("name", ["large", "small", "cluster_e0"])
@pytest.mark.parametrize("element,nchild", [("astro2", 8), ("astro", 4)])
def test_barnes_hut_reference_lists(oracle_mod, name, element, nchild):
    """Leaf 1 + exact traversal (the plugin's default) against the reference
    restatement at theta 0.5."""
    import physim_gb300 as pg
    _, m, spacing, e = _case(name)
    s = jittered_grid(m, spacing, seed=m + 2)
    acc = pg.accelerations(len(s))
    with pg.TransformElementHandler(element, {"theta": 0.5, "e": e}) as el:
        el.transform(s, acc)
    want = oracle_mod.barnes_hut(s, 0.5, e, nchild=nchild)
    err = rel_err(acc, want)
    assert err.max() < RTOL, (name, element, err.max())


@pytest.mark.parametrize("name", ["large", "small"])
def test_barnes_hut_warp_traversal_accuracy(oracle_mod, name):
    """Leaf 16 + warp traversal is never less accurate than the reference
    algorithm against the f64 direct sum (it opens every cell some body of
    the warp would open)."""
    import physim_gb300 as pg
    _, m, spacing, e = _case(name)
    s = jittered_grid(m, spacing, seed=m + 3)
    acc = pg.accelerations(len(s))
    props = {"theta": 0.7, "e": e, "leaf_size": 16, "traversal": "warp"}
    with pg.TransformElementHandler("astro2", props) as el:
        el.transform(s, acc)
    direct = oracle_mod.simple_astro(s, e)
    ref = oracle_mod.barnes_hut(s, 0.7, e, nchild=8)
    got_rms = np.sqrt(np.mean(rel_err(acc, direct) ** 2))
    ref_rms = np.sqrt(np.mean(rel_err(ref, direct) ** 2))
    assert np.isfinite(got_rms) and got_rms <= ref_rms * 1.01 + 1e-6, (got_rms, ref_rms)


def test_ensemble_members_at_far_scales(oracle_mod):
    """Members of 1e7, 1e-7 and 1e-6 scales in one ensemble, one of them
    (17,578 bodies) on the each-pair-once units: the first (Taylor) step's
    velocity change is a dt, so v / dt recovers each member's accelerations;
    then four more steps against the oracle pipeline (the pair scale follows
    the positions from step to step)."""
    import physim_gb300 as pg
    from test_verlet_gpu import trajectory_errors
    dt = 1e-3
    members = [jittered_grid(12, 2e6, seed=11, mass_scale=1e20),
               jittered_grid(12, 2e-8, seed=12, mass_scale=1e-30),
               jittered_grid(10, 1e-6, seed=13, mass_scale=1e-20),
               jittered_grid(26, 2e6, seed=14, mass_scale=1e20)]
    es = [0.01, 0.0, 0.0, 0.01]
    with pg.Ensemble(members, pg.SimConfig(gravity="simple_astro", e=0.01, dt=dt)) as ens:
        for k, e in enumerate(es):
            ens.set_member(k, e, dt)
        ens.step(1)
        first = [ens.download(k) for k in range(len(members))]
        ens.step(4)
        last = [ens.download(k) for k in range(len(members))]
    for k, (s, e) in enumerate(zip(members, es)):
        a = pg.accelerations(len(s))
        a["x"], a["y"], a["z"] = first[k]["vx"] / dt, first[k]["vy"] / dt, first[k]["vz"] / dt
        err = rel_err(a, oracle_mod.simple_astro(s, e))
        assert err.max() < RTOL, (k, err.max())
        want = oracle_mod.run_pipeline(s, "simple_astro", 5, dt, e)
        terr = trajectory_errors(s, last[k], want)
        assert terr["vel_rel_l2"] < 1e-5 and terr["pos_rel_l2"] < 1e-5, (k, terr)


@pytest.mark.parametrize("mass_scale", [1e33, 1e-33])
def test_extreme_masses_with_coincident_bodies(oracle_mod, mass_scale):
    """A pair at one position contributes 0 * m / sqrt(guard): masses are
    scaled by a power of two too, so that stays 0 (not 0 * inf = NaN) for
    masses up to the FP32 range, in both direct-sum plans and in Barnes-Hut
    (leaf 1, exact traversal), as the reference skips equal centres
    (transformers.rs:145,230)."""
    import physim_gb300 as pg
    s = jittered_grid(10, 0.05, seed=21, mass_scale=mass_scale)
    for k in range(3):  # a coincident group
        s[k]["x"], s[k]["y"], s[k]["z"] = s[500]["x"], s[500]["y"], s[500]["z"]
    want = oracle_mod.simple_astro(s, 0.01)
    acc = pg.accelerations(len(s))
    with pg.TransformElementHandler("simple_astro", {"e": 0.01}) as el:
        el.transform(s, acc)
    with pg.Simulation(s, pg.SimConfig(gravity="simple_astro", e=0.01)) as sim:
        sim.set_plan(symmetric=True)
        sym = sim.accelerations()
    bh = pg.accelerations(len(s))
    with pg.TransformElementHandler("astro2", {"theta": 0.5, "e": 0.01}) as el:
        el.transform(s, bh)
    want_bh = oracle_mod.barnes_hut(s, 0.5, 0.01, nchild=8)
    for got, ref in ((acc, want), (sym, want), (bh, want_bh)):
        assert np.isfinite(_vec(got)).all()
        assert rel_err(got, ref).max() < RTOL
