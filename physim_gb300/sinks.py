"""Render elements as host-side sinks: `csvsink` (utilities/src/csvsink.rs)
and `energysink` (debug/src/energysink.rs).

physim hands a renderer the initial state and the state after every step
(physim-core/src/pipeline.rs:130-181); csvsink writes state k when
k % print_n == 0 (csvsink.rs:44-70), one line per state: every entity's
`x,y,z,` then a newline (csvsink.rs:73-79), numbers in Rust's `{}` format for
f64 (the shortest decimal that reads back to the same value, never in
exponent notation: 1 -> "1", 1e-7 -> "0.0000001", -0.0 -> "-0").
"""
from __future__ import annotations

import ctypes as C
import math
import sys
from decimal import Decimal

import numpy as np


def rust_f64(v: float) -> str:
    """Rust's Display of an f64."""
    v = float(v)
    if math.isnan(v):
        return "NaN"
    if math.isinf(v):
        return "inf" if v > 0 else "-inf"
    if v == 0.0:
        return "-0" if math.copysign(1.0, v) < 0 else "0"
    s = format(Decimal(repr(v)), "f")
    if "." in s:
        s = s.rstrip("0").rstrip(".")
    return s


class CsvSink:
    """csvsink with properties `file` (default "csvsink.csv") and `print_n`
    (default 1)."""

    def __init__(self, file: str = "csvsink.csv", print_n: int = 1):
        self.file = file
        self.print_n = max(1, int(print_n))
        self.iteration = 0
        self._fh = open(file, "w", encoding="ascii", newline="")

    def render(self, state: np.ndarray, iteration: int | None = None) -> None:
        """Receives one state; `iteration` is its index in the sequence of
        states (counted here when not given)."""
        k = self.iteration if iteration is None else int(iteration)
        self.iteration = k + 1
        if k % self.print_n != 0:
            return
        parts = []
        for x, y, z in zip(state["x"].tolist(), state["y"].tolist(), state["z"].tolist()):
            parts.append(f"{rust_f64(x)},{rust_f64(y)},{rust_f64(z)},")
        self._fh.write("".join(parts) + "\n")

    def close(self) -> None:
        if self._fh and not self._fh.closed:
            self._fh.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class EnergySink:
    """physim's `energysink` (debug/src/energysink.rs) with its energy on the GPU.

    Every state it receives is reduced to the kinetic energy K and, once a
    gravity element has posted ("energysink", "gravity") (energysink.rs:
    112-117), the potential energy V, both in f64 on the device
    (physim_gpu_energy_compute); every `print_n`-th state prints the
    reference's line `{i:>5} :: K = .. :: V = .. :: E = .. :: Delta E ..`
    (energysink.rs:38-58; Delta E = E of the first state - E).  Two
    differences from the reference, both its bugs: V sums every pair (the
    reference assigns `=` where it means `+=`, energysink.rs:86, so it keeps
    the last pair only), and the first line's E is K + V (the reference
    prints V there).  With the default e = 0 the pair potential is the
    reference sink's -m_a m_b / r; with `e` > 0 it is the potential whose
    gradient is the softened force of the gravity elements.  `records` keeps
    (iteration, K, V, E, Delta E) of every state."""

    def __init__(self, print_n: int = 1, e: float = 0.0, device: int = 0, out=None):
        from ._lib import check, lib
        self.print_n = max(1, int(print_n))
        self.e = abs(float(e))
        self.calc_gpe = False
        self.iteration = 0
        self.initial_energy = None
        self.records: list[tuple[int, float, float, float, float]] = []
        self.out = out if out is not None else sys.stdout
        h = C.c_void_p()
        check(lib.physim_gpu_energy_create(device, C.byref(h)), "physim_gpu_energy_create")
        self.handle = h

    def recv_message(self, topic: str, message: str, priority: int = 2, sender: int = 0) -> None:
        if topic == "energysink" and message == "gravity":
            self.calc_gpe = True

    def energy(self, state: np.ndarray) -> tuple[float, float]:
        """(potential, kinetic) of one state."""
        from ._lib import PhysimDiagnostics, check, lib
        from .entity import as_entities
        state = as_entities(state)
        d = PhysimDiagnostics()
        check(lib.physim_gpu_energy_compute(self.handle, state.ctypes.data, len(state), self.e,
                                            1 if self.calc_gpe else 0, C.byref(d)),
              "physim_gpu_energy_compute")
        return (d.potential if self.calc_gpe else 0.0), d.kinetic

    def render(self, state: np.ndarray) -> None:
        potential, kinetic = self.energy(state)
        energy = kinetic + potential
        if self.initial_energy is None:
            self.initial_energy = energy
        delta = self.initial_energy - energy
        k = self.iteration
        self.iteration += 1
        self.records.append((k, kinetic, potential, energy, delta))
        if k == 0 or k % self.print_n == 0:
            self.out.write(f"{k:>5} :: K = {kinetic:.6f} :: V = {potential:.6f} :: "
                           f"E = {energy:.6f} :: Delta E {delta:.6f}\n")

    def close(self) -> None:
        from ._lib import lib
        if self.handle:
            lib.physim_gpu_energy_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
