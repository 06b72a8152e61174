"""The cube and plummer initialisers generated on the GPU against the
oracle's restatement with the same variates: cube bit for bit (only +, *,
/), plummer within 1e-14 relative (the device's sin, cos and pow against the
host's libm); a simulation initialised on the device holds the same bodies
and steps like an uploaded one; the csvsink writer on a device-resident run."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FIELDS = ("x", "y", "z", "vx", "vy", "vz", "radius", "mass", "id", "fixed")


@pytest.mark.parametrize("n", [1, 1000, 65537])
def test_cube_bit_exact(oracle_mod, n):
    from physim_gb300 import initialisers
    props = {"n": n, "seed": 11, "spin": 1.5, "size": 0.5, "centre": (0.1, -0.2, 0.3),
             "mass": 3.0, "id": 9}
    got = initialisers.cube(props)
    want = oracle_mod.cube(props)
    for f in FIELDS:
        assert got[f].tobytes() == want[f].tobytes(), f


def test_plummer_matches_oracle(oracle_mod):
    from physim_gb300 import initialisers
    props = {"n": 50000, "seed": 4, "mass": 2.0, "a": 0.2, "spin": 0.5,
             "centre": (1.0, 0.0, -1.0), "v": (0.0, 0.5, 0.0), "id": 2}
    got = initialisers.plummer(props)
    want = oracle_mod.plummer(props)
    for f in ("x", "y", "z", "vx", "vy", "vz"):
        np.testing.assert_allclose(got[f], want[f], rtol=1e-14, atol=1e-15, err_msg=f)
    for f in ("radius", "mass", "id", "fixed"):
        assert got[f].tobytes() == want[f].tobytes(), f


@pytest.mark.parametrize("kind", ["cube", "plummer"])
def test_generated_simulation(oracle_mod, kind):
    """Simulation.generated holds the generator's bodies and steps exactly as
    the same bodies uploaded."""
    import physim_gb300 as pg
    from physim_gb300 import initialisers
    props = {"n": 3000, "seed": 21, "spin": 0.3}
    cfg = pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)
    bodies = initialisers.cube(props) if kind == "cube" else initialisers.plummer(props)
    with pg.Simulation.generated(kind, props, cfg) as a, pg.Simulation(bodies, cfg) as b:
        s0 = a.download()
        for f in FIELDS:
            assert s0[f].tobytes() == bodies[f].tobytes(), f
        a.step(5)
        b.step(5)
        sa, sb = a.download(), b.download()
    for f in FIELDS:
        assert sa[f].tobytes() == sb[f].tobytes(), f


def test_csvsink_on_device_run(tmp_path):
    """Simulation.run with a csvsink: the initial state and every print_n-th
    step, each line the entities' x,y,z in Rust's f64 format."""
    import physim_gb300 as pg
    from physim_gb300.sinks import CsvSink, rust_f64
    props = {"n": 50, "seed": 3}
    cfg = pg.SimConfig(gravity="simple_astro", e=0.01, dt=1e-5)
    path = tmp_path / "run.csv"
    with pg.Simulation.generated("cube", props, cfg) as sim, CsvSink(str(path), print_n=4) as sink:
        sim.run(10, sink=sink)
        last = sim.download()
    lines = path.read_text().splitlines()
    assert len(lines) == 3  # states 0, 4, 8
    with pg.Simulation.generated("cube", props, cfg) as sim:
        sim.step(8)
        s8 = sim.download()
    want = "".join(f"{rust_f64(x)},{rust_f64(y)},{rust_f64(z)},"
                   for x, y, z in zip(s8["x"], s8["y"], s8["z"]))
    assert lines[2] == want
    assert not np.array_equal(last["x"], s8["x"])
