"""Entity / Acceleration arrays with physim's C layout (physim-core/src/lib.rs:16-37).

`ENTITY` is the numpy dtype of physim's repr(C) Entity (80 bytes: eight f64,
a usize id at offset 64, a bool `fixed` at 72, 7 bytes of padding), so a
numpy array of it can be handed to the C ABI as `const Entity*` unchanged.
"""
from __future__ import annotations

import numpy as np

ENTITY = np.dtype({
    "names": ["x", "y", "z", "vx", "vy", "vz", "radius", "mass", "id", "fixed"],
    "formats": ["<f8"] * 8 + ["<u8", "u1"],
    "offsets": [0, 8, 16, 24, 32, 40, 48, 56, 64, 72],
    "itemsize": 80,
})
ACCELERATION = np.dtype({"names": ["x", "y", "z"], "formats": ["<f8"] * 3, "offsets": [0, 8, 16],
                         "itemsize": 24})


def as_entities(a: np.ndarray) -> np.ndarray:
    """`a` as a C-contiguous array of exactly ENTITY (80-byte records).

    numpy drops the padding of structured dtypes in some operations (e.g.
    np.concatenate returns packed 73-byte records); such arrays are converted
    field by field so the C ABI always sees physim's layout."""
    a = np.asarray(a)
    if a.dtype != ENTITY or a.dtype.itemsize != 80:
        a = a.astype(ENTITY)
    return np.ascontiguousarray(a)


def as_accelerations(a: np.ndarray) -> np.ndarray:
    a = np.asarray(a)
    if a.dtype != ACCELERATION or a.dtype.itemsize != 24:
        a = a.astype(ACCELERATION)
    return np.ascontiguousarray(a)


def entities(n: int) -> np.ndarray:
    """A zeroed Entity array (Entity::default(), physim-core/src/lib.rs:16)."""
    return np.zeros(n, dtype=ENTITY)


def accelerations(n: int) -> np.ndarray:
    """A zeroed Acceleration array (Acceleration::zero(), lib.rs:40-46)."""
    return np.zeros(n, dtype=ACCELERATION)


def entity_new(x: float, y: float, z: float, mass: float) -> np.void:
    """Entity::new (physim-core/src/lib.rs:94-103): radius = mass^0.33333."""
    e = np.zeros((), dtype=ENTITY)
    e["x"], e["y"], e["z"], e["mass"] = x, y, z, mass
    e["radius"] = mass ** 0.33333
    return e


def positions(state: np.ndarray) -> np.ndarray:
    return np.stack([state["x"], state["y"], state["z"]], axis=1)


def acc_array(acc: np.ndarray) -> np.ndarray:
    return np.stack([acc["x"], acc["y"], acc["z"]], axis=1)


def from_arrays(pos: np.ndarray, vel: np.ndarray | None, mass: np.ndarray,
                fixed: np.ndarray | None = None, radius: np.ndarray | None = None,
                ids: np.ndarray | None = None) -> np.ndarray:
    n = len(mass)
    s = entities(n)
    s["x"], s["y"], s["z"] = pos[:, 0], pos[:, 1], pos[:, 2]
    if vel is not None:
        s["vx"], s["vy"], s["vz"] = vel[:, 0], vel[:, 1], vel[:, 2]
    s["mass"] = mass
    if radius is not None:
        s["radius"] = radius
    if ids is not None:
        s["id"] = ids
    if fixed is not None:
        s["fixed"] = fixed.astype(np.uint8)
    return s
