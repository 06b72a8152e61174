"""The `cube` and `plummer` initialiser elements (astro/src/initialisers.rs)
generated on the GPU (physim_gpu_generate_* / physim_gpu_sim_init_*).

Properties and defaults are the reference's (initialisers.rs:35-80 for cube,
:233-284 for plummer).  The uniform variates are this library's counter-based
stream (SplitMix64 of the seed and the body index), not the reference's
ChaCha8 stream, so a given seed gives different bodies than physim does, drawn
from the same distributions with the same formulas.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import PhysimCubeParams, PhysimPlummerParams, check, lib
from .entity import ENTITY

CUBE_DEFAULTS = {"n": 100_000, "seed": 0, "spin": 0.0, "size": 1.0, "centre": (0.0, 0.0, 0.0),
                 "mass": 1.0, "id": 0}
PLUMMER_DEFAULTS = {"n": 100_000, "seed": 0, "mass": 1.0, "a": 1.0, "centre": (0.0, 0.0, 0.0),
                    "v": (0.0, 0.0, 0.0), "spin": 0.0, "id": 0}


def cube_params(props: dict | None = None) -> tuple[int, PhysimCubeParams]:
    q = {**CUBE_DEFAULTS, **(props or {})}
    p = PhysimCubeParams(int(q["seed"]), float(q["spin"]), float(q["size"]), float(q["mass"]),
                         (C.c_double * 3)(*q["centre"]), int(q["id"]))
    return int(q["n"]), p


def plummer_params(props: dict | None = None) -> tuple[int, PhysimPlummerParams]:
    q = {**PLUMMER_DEFAULTS, **(props or {})}
    p = PhysimPlummerParams(int(q["seed"]), float(q["mass"]), float(q["a"]), float(q["spin"]),
                            (C.c_double * 3)(*q["centre"]), (C.c_double * 3)(*q["v"]),
                            int(q["id"]))
    return int(q["n"]), p


def cube(props: dict | None = None, device: int = 0) -> np.ndarray:
    """`cube` bodies as a host Entity array."""
    n, p = cube_params(props)
    out = np.zeros(n, dtype=ENTITY)
    check(lib.physim_gpu_generate_cube(C.byref(p), out.ctypes.data, n, device),
          "physim_gpu_generate_cube")
    return out


def plummer(props: dict | None = None, device: int = 0) -> np.ndarray:
    """`plummer` bodies as a host Entity array."""
    n, p = plummer_params(props)
    out = np.zeros(n, dtype=ENTITY)
    check(lib.physim_gpu_generate_plummer(C.byref(p), out.ctypes.data, n, device),
          "physim_gpu_generate_plummer")
    return out
