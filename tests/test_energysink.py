"""The energysink counterpart (debug/src/energysink.rs) and the message path
that turns its potential on: a gravity element's configuration message
("energysink", "gravity") (transformers.rs:107-111,198-203,266-270) reaches
the sink through the host's message bus (messages.rs:201-271).

CPU: the library posts the message through the bus mirror and it is
delivered to every client.  GPU: K and V of each state against numpy f64
(relative 1e-6: pair terms are FP32, all sums f64), V only after the message
arrived, and the reference's output line."""
from __future__ import annotations

import io

import numpy as np
import pytest


class _Client:
    def __init__(self):
        self.got = []

    def recv_message(self, topic, message, priority=2, sender=0):
        self.got.append((topic, message, priority))


@pytest.mark.parametrize("element", ["astro", "astro2", "simple_astro"])
def test_configuration_message_delivered_through_bus(element):
    import physim_gb300 as pg
    from physim_gb300.plugin import MessageBus
    client = _Client()
    with pg.TransformElementHandler(element, {"e": 0.1}) as el:
        with MessageBus() as bus:
            el.post_configuration_messages()
        assert bus.deliver([client]) == 1
    assert client.got == [("energysink", "gravity", 1)]  # MessagePriority::Low
    (prio, topic, message, _, origin), = bus.messages
    assert (prio, topic, message, origin) == (1, "energysink", "gravity", 1)  # origin C


def test_no_bus_installed_posts_nothing():
    """Outside a bus (and without physim's post_bus_callback) the message is
    dropped, as the library does when physim's bus is absent."""
    import physim_gb300 as pg
    from physim_gb300.plugin import MessageBus
    with MessageBus() as bus:
        pass
    with pg.TransformElementHandler("astro2", {}) as el:
        el.post_configuration_messages()
    assert bus.messages == []


def _energies(state, e):
    m = state["mass"]
    v2 = state["vx"] ** 2 + state["vy"] ** 2 + state["vz"] ** 2
    kin = float(np.sum(0.5 * m * v2))
    p = np.stack([state["x"], state["y"], state["z"]], 1)
    pot = 0.0
    for i in range(len(state) - 1):
        r = np.linalg.norm(p[i + 1:] - p[i], axis=1)
        phi = np.arctan(np.sqrt(e) / r) / np.sqrt(e) if e > 0 else 1.0 / r
        pot -= float(np.sum(m[i] * m[i + 1:] * phi))
    return kin, pot


@pytest.mark.gpu
@pytest.mark.parametrize("e", [0.0, 0.01])
def test_energysink_in_a_pipeline(e):
    import physim_gb300 as pg
    from physim_gb300 import ics
    from physim_gb300.sinks import EnergySink
    s = ics.cube_with_stars(1500, seed=31, stars=ics.STARS_2)
    out = io.StringIO()
    el = pg.TransformElementHandler("astro2", {"theta": 0.5, "e": 0.01})
    sink = EnergySink(print_n=2, e=e, out=out)
    states = []

    class Keep:
        def recv_message(self, *a, **k):
            pass

        def render(self, st):
            states.append(st.copy())

    pipe = pg.Pipeline([el], pg.GpuVerlet(), 1e-5, sinks=[sink, Keep()])
    pipe.run(s, 3)
    assert sink.calc_gpe and len(sink.records) == 4 == len(states)
    for (k, kin, pot, energy, delta), st in zip(sink.records, states):
        want_k, want_v = _energies(st, e)
        assert kin == pytest.approx(want_k, rel=1e-6)
        assert pot == pytest.approx(want_v, rel=1e-6) and pot < 0.0
        assert energy == pytest.approx(kin + pot, rel=1e-12)
        assert delta == pytest.approx(sink.records[0][3] - energy, abs=1e-9 * abs(energy))
    lines = out.getvalue().splitlines()
    assert [ln.split(" :: ")[0].strip() for ln in lines] == ["0", "2"]
    assert lines[0].startswith("    0 :: K = ") and " :: Delta E " in lines[0]
    sink.close()
    el.destroy()


@pytest.mark.gpu
def test_energysink_without_gravity_reports_kinetic_only():
    import physim_gb300 as pg
    from physim_gb300 import ics
    from physim_gb300.sinks import EnergySink
    s = ics.cube_with_stars(200, seed=32)
    with EnergySink(out=io.StringIO()) as sink:
        sink.render(s)
        assert not sink.calc_gpe
        (_, kin, pot, _, _), = sink.records
    assert pot == 0.0 and kin == pytest.approx(_energies(s, 0.0)[0], rel=1e-12)
