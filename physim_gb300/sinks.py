"""The `csvsink` render element (utilities/src/csvsink.rs) as a host-side writer.

physim hands a renderer the initial state and the state after every step
(physim-core/src/pipeline.rs:130-181); csvsink writes state k when
k % print_n == 0 (csvsink.rs:44-70), one line per state: every entity's
`x,y,z,` then a newline (csvsink.rs:73-79), numbers in Rust's `{}` format for
f64 (the shortest decimal that reads back to the same value, never in
exponent notation: 1 -> "1", 1e-7 -> "0.0000001", -0.0 -> "-0").
"""
from __future__ import annotations

import math
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
