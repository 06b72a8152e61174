"""Writes the golden fixtures the CPU tests check the oracle against.

  tree_kats.json   the reference's own tree tests (astro/src/octree.rs:218-519,
                   astro/src/quadtree.rs:197-492) as data: tree kind, root box,
                   bodies (listed or as a seeded generator), queries, and the
                   leaf count or relation each test asserts.  Tests that draw
                   bodies from rand_chacha streams (not vendored) use a PCG64
                   stream over the same ranges; every such assertion holds for
                   any stream with distinct positions.
  law_kats.json    analytic known answers of the force law
                   (astro/src/lib.rs:84-113) on Pythagorean separations, with
                   exact rational values, and of small direct sums.
  oracle_fixtures.npz  regression pins of the oracle itself on small seeded
                   states (simple_astro, astro2, astro, verlet), produced by
                   running oracle/ (so a later edit that changes its
                   arithmetic is caught).

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import sys
from fractions import Fraction
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))


def ent(x, y, z, m):
    return {"x": x, "y": y, "z": z, "mass": m}


def tree_kats() -> list[dict]:
    k = []
    for kind, nchild in (("octree", 8), ("quadtree", 4)):
        def add(name, extent, bodies, queries, centre=(0.0, 0.0, 0.0)):
            k.append({"tree": kind, "nchild": nchild, "name": name, "centre": list(centre),
                      "extent": extent, "bodies": bodies, "queries": queries})
        add("test_empty_tree", 1.0, [], [{"loc": [0, 0, 0], "theta": 0.5, "eq": 0}])
        add("test_single_entity", 1.0, [ent(0, 0, 0, 1.0)],
            [{"loc": [0, 0, 0], "theta": 0.5, "eq": 1}])
        add("test_entities_at_origin", 2.0, [ent(0, 0, 0, 1.0)] * 10,
            [{"loc": [0, 0, 0], "theta": 0.5, "eq": 1}])
        if nchild == 8:
            pos = [[0.5, 0.5, 0.5], [-0.5, 0.5, 0.5], [0.5, -0.5, 0.5], [-0.5, -0.5, 0.5],
                   [0.5, 0.5, -0.5], [-0.5, 0.5, -0.5], [0.5, -0.5, -0.5], [-0.5, -0.5, -0.5]]
            add("test_entities_in_different_octants", 2.0, [ent(*p, 1.0) for p in pos],
                [{"loc": [0, 0, 0], "theta": 0.5, "eq": 8}])
        else:
            pos = [[0.5, 0.5, 0.5], [-0.5, 0.5, 0.5], [0.5, -0.5, 0.5], [-0.5, -0.5, 0.5]]
            add("test_entities_in_different_quadrants", 2.0, [ent(*p, 1.0) for p in pos],
                [{"loc": [0, 0, 0], "theta": 0.5, "eq": 4}])
        add("test_bh_factor_filtering", 10.0,
            [ent(0.1, 0, 0, 1.0), ent(5.0, 0, 0, 1.0), ent(8.0, 0, 0, 1.0)],
            [{"loc": [0, 0, 0], "theta": -0.1, "eq": 3},
             {"loc": [0, 0, 0], "theta": 1.0, "gt": 0}])
        if nchild == 8:
            b = [ent(1.0, 0, 0, 1.0), ent(-1.0, 0, 0, 1.0), ent(0, 1.0, 0, 1.0),
                 ent(0, -1.0, 0, 1.0), ent(0, 0, 1.0, 1.0), ent(0, 0, -1.0, 1.0)]
            add("test_boundary_conditions", 1.0, b, [{"loc": [0, 0, 0], "theta": -0.1, "eq": 6}])
        else:
            b = [ent(1.0, 0, 0, 1.0), ent(-1.0, 0, 0, 1.0), ent(0, 1.0, 0, 1.0),
                 ent(0, -1.0, 0, 1.0)]
            add("test_boundary_conditions", 1.0, b, [{"loc": [0, 0, 0], "theta": -0.1, "eq": 4}])
        add("test_query_from_different_locations", 10.0,
            [ent(i * 0.1, 0, 0, 1.0) for i in range(20)],
            [{"loc": [0, 0, 0], "theta": 0.5, "gt": 0},
             {"loc": [100.0, 0, 0], "theta": 0.5, "gt": 0}])
        add("test_dense_cluster", 1.0, {"gen": "cluster", "seed": 42, "n": 1000, "scale": 0.2},
            [{"loc": [0, 0, 0], "theta": -0.1, "eq": 1000}])
        add("test_sparse_distribution", 100.0,
            {"gen": "cluster", "seed": 123, "n": 100, "scale": 200.0},
            [{"loc": [0, 0, 0], "theta": -0.1, "eq": 100}])
        add("test_resolution_threshold", 10.0,
            [ent(1.0, 0, 0, 1.0), ent(5.0, 0, 0, 1.0), ent(9.0, 0, 0, 1.0)],
            [{"loc": [0, 0, 0], "theta": 0.1, "label": "loose"},
             {"loc": [0, 0, 0], "theta": 0.5, "label": "medium"},
             {"loc": [0, 0, 0], "theta": 2.0, "label": "strict"}])
        add("test_lots", 1.0, {"gen": "random", "seed": 0, "n": 100_000},
            [{"loc": [0, 0, 0], "theta": -0.1, "eq": 100_000}])
        add("test_extreme_coordinates", 1000.0,
            [ent(999.0, 999.0, 999.0, 1.0), ent(-999.0, -999.0, -999.0, 1.0)],
            [{"loc": [0, 0, 0], "theta": -0.1, "eq": 2}])
        add("test_zero_extent", 0.001, [ent(0, 0, 0, 1.0)],
            [{"loc": [0, 0, 0], "theta": -0.1, "eq": 1}])
        add("test_query_outside_bounds", 1.0, [ent(0, 0, 0, 1.0)],
            [{"loc": [1000.0, 1000.0, 1000.0], "theta": 0.5, "gt": 0}])
        add("test_reproducibility", 1.0, {"gen": "random", "seed": 999, "n": 1000},
            [{"loc": [0, 0, 0], "theta": -0.1, "same_as_rebuild": True}])
    return k


def _sqrt_exact(q: Fraction) -> Fraction:
    num, den = q.numerator, q.denominator
    rn, rd = int(round(num ** 0.5)), int(round(den ** 0.5))
    assert rn * rn == num and rd * rd == den
    return Fraction(rn, rd)


def law_kats() -> dict:
    """F = (b - a)/r * m_a m_b / (r^2 + e) with r a whole number."""
    cases = []
    specs = [((0, 0, 0), 2, (3, 4, 0), 5, 1), ((0, 0, 0), 1, (1, 2, 2), 1, 0),
             ((1, 1, 1), 3, (3, 4, 7), 0.5, Fraction(1, 4)), ((-2, 5, 1), 7, (0, 8, 7), 11, 2),
             ((0.5, 0.5, 0.5), 1, (0.5, 0.5, 3.5), 1e5, Fraction(1, 100))]
    for a, ma, b, mb, e in specs:
        A = [Fraction(v) for v in a]
        B = [Fraction(v) for v in b]
        ma_f, mb_f, e_f = Fraction(ma), Fraction(mb), Fraction(e)
        d2 = sum((bb - aa) ** 2 for aa, bb in zip(A, B))
        r = _sqrt_exact(d2)
        f = [(bb - aa) / r * ma_f * mb_f / (d2 + e_f) for aa, bb in zip(A, B)]
        cases.append({"a": [float(v) for v in A], "ma": float(ma_f), "b": [float(v) for v in B],
                      "mb": float(mb_f), "e": float(e_f), "force": [float(v) for v in f]})
    # A direct sum on three bodies: acc of body 0 = sum_j F_0j / m_0.
    bodies = [((0, 0, 0), 2), ((3, 4, 0), 5), ((0, 0, 12), 3)]
    e = Fraction(1)
    A = [Fraction(v) for v in bodies[0][0]]
    acc = [Fraction(0)] * 3
    for pos, m in bodies[1:]:
        B = [Fraction(v) for v in pos]
        d2 = sum((bb - aa) ** 2 for aa, bb in zip(A, B))
        r = _sqrt_exact(d2)
        for c in range(3):
            acc[c] += (B[c] - A[c]) / r * bodies[0][1] * m / (d2 + e) / bodies[0][1]
    return {"pairs": cases,
            "direct3": {"bodies": [[*map(float, p), float(m)] for p, m in bodies], "e": 1.0,
                        "acc0": [float(v) for v in acc]}}


def _zero_padding(a: np.ndarray) -> np.ndarray:
    """The same records with zero struct padding (the oracle copies whole C
    structs, whose padding bytes are unspecified), so that the fixture file
    regenerates byte for byte."""
    out = np.zeros(a.shape, a.dtype)
    for name in a.dtype.names:
        out[name] = a[name]
    return out


def oracle_fixtures(path: Path) -> None:
    import oracle
    from physim_gb300.entity import ACCELERATION, ENTITY  # noqa: F401 (dtype only)
    from physim_gb300 import ics

    st = ics.cube_with_stars(253, seed=5, stars=ics.STARS_2)
    st["fixed"][3] = 1
    acc_direct = oracle.simple_astro(st, 0.01)
    acc_oct = oracle.barnes_hut(st, 0.5, 0.01, nchild=8)
    acc_quad = oracle.barnes_hut(st, 0.7, 0.01, nchild=4)
    traj = _zero_padding(oracle.run_pipeline(st, "simple_astro", 3, 1e-5, 0.01))
    traj_bh = _zero_padding(oracle.run_pipeline(st, "astro2", 3, 1e-5, 0.01, theta=1.0))
    np.savez_compressed(path, state=st.view(np.uint8), acc_direct=acc_direct.view(np.uint8),
                        acc_octree=acc_oct.view(np.uint8), acc_quadtree=acc_quad.view(np.uint8),
                        traj_direct=traj.view(np.uint8), traj_astro2=traj_bh.view(np.uint8))


def main() -> None:
    (HERE / "tree_kats.json").write_text(json.dumps(tree_kats(), indent=1) + "\n")
    (HERE / "law_kats.json").write_text(json.dumps(law_kats(), indent=1) + "\n")
    oracle_fixtures(HERE / "oracle_fixtures.npz")
    print("wrote", *(p.name for p in sorted(HERE.iterdir()) if p.suffix in (".json", ".npz")))


if __name__ == "__main__":
    main()
