"""The csvsink writer (utilities/src/csvsink.rs) and the oracle's restatement
of the cube / plummer initialisers (astro/src/initialisers.rs).  CPU only."""
from __future__ import annotations

import math

import numpy as np
import pytest


def test_rust_f64_display():
    """Rust's `{}` for f64: shortest round-trip digits, never exponent
    notation, integers without a fraction, "-0", "NaN", "inf"."""
    from physim_gb300.sinks import rust_f64
    cases = [(1.0, "1"), (0.1, "0.1"), (-2.5, "-2.5"), (1e-7, "0.0000001"),
             (1.5e20, "150000000000000000000"), (123.456, "123.456"), (-0.0, "-0"), (0.0, "0"),
             (math.inf, "inf"), (-math.inf, "-inf"),
             (0.30000000000000004, "0.30000000000000004"), (2.0 ** 60, "1152921504606847000")]
    for v, want in cases:
        assert rust_f64(v) == want, (v, rust_f64(v))
    assert rust_f64(float("nan")) == "NaN"
    assert rust_f64(5e-324) == "0." + "0" * 323 + "5"
    for v in np.random.default_rng(1).normal(0, 1e3, 200):
        assert float(rust_f64(v)) == v  # round trip


def test_csvsink_lines_and_print_n(tmp_path):
    """One line per printed state: `x,y,z,` per entity; states k with
    k % print_n == 0, counting from the initial state (csvsink.rs:44-79)."""
    from physim_gb300.entity import entities
    from physim_gb300.sinks import CsvSink
    s = entities(2)
    s["x"], s["y"], s["z"] = [1.0, 0.5], [-0.0, 2.0], [1e-7, 3.0]
    path = tmp_path / "out.csv"
    with CsvSink(str(path), print_n=2) as sink:
        for k in range(5):
            t = s.copy()
            t["x"] += k
            sink.render(t)
    lines = path.read_text().splitlines()
    assert lines == ["1,-0,0.0000001,0.5,2,3,", "3,-0,0.0000001,2.5,2,3,",
                     "5,-0,0.0000001,4.5,2,3,"]


def test_oracle_cube_formulas(oracle_mod):
    """initialisers.rs:81-106: positions in [-size, size)^2 x [0, size) about
    the centre, v = (y, -x, 0) * spin of the scaled position, mass = total / n,
    radius 0.02 (Entity::random)."""
    props = {"n": 20000, "seed": 5, "spin": 3.0, "size": 2.0, "centre": (1.0, -1.0, 0.5),
             "mass": 7.0, "id": 4}
    c = oracle_mod.cube(props)
    x, y, z = c["x"] - 1.0, c["y"] + 1.0, c["z"] - 0.5
    assert x.min() >= -2.0 and x.max() < 2.0 and y.min() >= -2.0 and y.max() < 2.0
    assert z.min() >= 0.0 and z.max() < 2.0 and abs(z.mean() - 1.0) < 0.02
    np.testing.assert_allclose(c["vx"], y * 3.0, rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(c["vy"], -x * 3.0, rtol=1e-12, atol=1e-12)
    assert np.all(c["vz"] == 0.0) and np.all(c["mass"] == 7.0 / 20000)
    assert np.all(c["radius"] == 0.02) and np.all(c["id"] == 4) and not c["fixed"].any()
    again = oracle_mod.cube(props)
    assert again.tobytes() == c.tobytes()  # deterministic in the seed
    other = oracle_mod.cube({**props, "seed": 6})
    assert not np.array_equal(other["x"], c["x"])


def test_oracle_plummer_formulas(oracle_mod):
    """initialisers.rs:286-330 as written: r = a (c^(-2/3) - 1)^(1/2) (the
    reciprocal of the Plummer profile's inverse mass function, so the median
    radius is a (0.5^(-2/3) - 1)^(1/2) = 0.766 a, not the profile's 1.305 a),
    theta = pi c (uniform, not isotropic), tangential speed
    spin sqrt(M r^2 / (r^2 + a^2)^1.5) plus the bulk velocity, radius 0.01."""
    a, M, spin = 0.3, 2.0, 0.7
    p = oracle_mod.plummer({"n": 100000, "seed": 2, "a": a, "mass": M, "spin": spin,
                            "v": (1.0, 0.0, -2.0)})
    r = np.sqrt(p["x"] ** 2 + p["y"] ** 2 + p["z"] ** 2)
    assert abs(np.median(r) / (a * math.sqrt(0.5 ** (-2 / 3) - 1)) - 1) < 0.01
    theta = np.arccos(np.clip(p["z"] / r, -1, 1))
    assert abs(np.median(theta) - math.pi / 2) < 0.01
    assert abs(np.mean(theta < math.pi / 4) - 0.25) < 0.01  # uniform in theta
    vt = np.sqrt((p["vx"] - 1.0) ** 2 + p["vy"] ** 2)
    np.testing.assert_allclose(vt, spin * np.sqrt(M * r ** 2 / (r ** 2 + a * a) ** 1.5),
                               rtol=1e-9)
    assert np.all(p["vz"] == -2.0) and np.all(p["radius"] == 0.01)
    assert np.all(p["mass"] == M / 100000)
