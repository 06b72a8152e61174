"""CPU oracle for physim's gravity + integration hot path -- TEST INFRASTRUCTURE.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg use this
package: as the reference the CUDA results are compared with, or as the timed
CPU baseline.  The shipped library never loads it.

`physim_oracle.c` restates the reference's Rust algorithms in C (f64, same
operation order); see its header for the file:line of each function and for
the parity status.  `bh_model.c` is the CPU model of the GPU Barnes-Hut
build (keys, sort order, tree), used for bit-exact checks of the GPU tree.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB = BUILD / "liboracle.so"
SOURCES = [HERE / "physim_oracle.c"] + sorted(p for p in HERE.glob("bh_model.c"))
CFLAGS = ["-O3", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11", "-Wall",
          "-Wextra", "-Wno-unused-parameter"]


def build(force: bool = False) -> Path:
    """Compiles the oracle with gcc (no -march flags: the same source runs on
    x86_64 and aarch64 hosts)."""
    BUILD.mkdir(exist_ok=True)
    if not force and LIB.exists() and all(s.stat().st_mtime <= LIB.stat().st_mtime
                                           for s in SOURCES):
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [os.environ.get("CC", "gcc"), *CFLAGS, "-o", str(tmp), *map(str, SOURCES), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"oracle build failed: {' '.join(cmd)}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


_lib = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = C.CDLL(str(LIB))
    vp, sz, dbl, i32 = C.c_void_p, C.c_size_t, C.c_double, C.c_int
    d3 = C.POINTER(C.c_double)
    sig = {
        "oracle_sizeof_entity": (i32, []),
        "oracle_sizeof_acceleration": (i32, []),
        "oracle_law": (None, [vp, vp, dbl, d3]),
        "oracle_tree_new": (vp, [i32, d3, dbl]),
        "oracle_tree_free": (None, [vp]),
        "oracle_tree_push": (i32, [vp, vp]),
        "oracle_tree_leaves": (sz, [vp, d3, dbl, vp, sz]),
        "oracle_tree_node_count": (sz, [vp]),
        "oracle_simple_astro": (None, [vp, sz, dbl, vp]),
        "oracle_simple_astro_sample": (None, [vp, sz, dbl, vp, sz, vp, i32]),
        "oracle_barnes_hut": (i32, [i32, vp, sz, dbl, dbl, vp, sz, vp, i32]),
        "oracle_astro2": (i32, [vp, sz, dbl, dbl, vp]),
        "oracle_astro": (i32, [vp, sz, dbl, dbl, vp]),
        "oracle_state_extent": (dbl, [vp, sz]),
        "oracle_verlet_new": (vp, []),
        "oracle_verlet_free": (None, [vp]),
        "oracle_verlet_step": (i32, [vp, vp, vp, sz, vp, dbl]),
        "oracle_run_pipeline": (i32, [vp, sz, i32, dbl, dbl, dbl, i32, i32]),
        "oracle_run_pipeline_with": (i32, [vp, sz, i32, i32, dbl, dbl, dbl, i32, i32]),
        "oracle_euler_step": (None, [vp, vp, sz, vp, dbl]),
        "oracle_rk4_step": (i32, [vp, vp, sz, vp, vp, dbl]),
        "oracle_max_threads": (i32, []),
        "oracle_tree_dump": (sz, [vp, vp, vp, sz]),
        "bh_model_extent": (dbl, [vp, sz]),
        "bh_model_keys": (None, [vp, sz, i32, vp]),
        "bh_model_build": (C.c_long, [vp, sz, i32, i32, vp, vp, vp, vp, vp, vp, vp, vp, sz]),
        "bh_model_accel": (i32, [vp, sz, i32, i32, dbl, dbl, i32, dbl, vp, sz, vp]),
        "oracle_cube": (None, [C.c_uint64, dbl, dbl, dbl, d3, C.c_uint64, sz, vp]),
        "oracle_plummer": (None, [C.c_uint64, dbl, dbl, dbl, d3, d3, C.c_uint64, sz, vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


# ---------------------------------------------------------------------------
# numpy-level helpers (arrays use physim_gb300.entity.ENTITY / ACCELERATION)
# ---------------------------------------------------------------------------
def _entity_dtype():
    from physim_gb300.entity import ACCELERATION, ENTITY
    return ENTITY, ACCELERATION


def _ent(a):
    from physim_gb300.entity import as_entities
    return as_entities(a)


def _acc(a):
    from physim_gb300.entity import as_accelerations
    return as_accelerations(a)


def law(a, b, e: float) -> np.ndarray:
    lib = load()
    out = (C.c_double * 3)()
    ENTITY, _ = _entity_dtype()
    aa = np.array(a, dtype=ENTITY)
    bb = np.array(b, dtype=ENTITY)
    lib.oracle_law(aa.ctypes.data, bb.ctypes.data, e, out)
    return np.array(list(out))


def simple_astro(state: np.ndarray, e: float, acc: np.ndarray | None = None) -> np.ndarray:
    """`+=` the reference simple_astro accelerations into acc (serial)."""
    lib = load()
    _, ACC = _entity_dtype()
    state = _ent(state)
    if acc is None:
        acc = np.zeros(len(state), dtype=ACC)
    if acc.dtype != ACC or not acc.flags.c_contiguous:
        raise TypeError("acc must be a C-contiguous ACCELERATION array")
    lib.oracle_simple_astro(state.ctypes.data, len(state), e, acc.ctypes.data)
    return acc


def simple_astro_sample(state: np.ndarray, e: float, idx: np.ndarray, threads: int = 0) -> np.ndarray:
    """Reference simple_astro accelerations of the bodies idx (f64 direct sum)."""
    lib = load()
    _, ACC = _entity_dtype()
    state = _ent(state)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.zeros(len(idx), dtype=ACC)
    lib.oracle_simple_astro_sample(state.ctypes.data, len(state), e, idx.ctypes.data, len(idx),
                                   out.ctypes.data, threads)
    return out


def barnes_hut(state: np.ndarray, theta: float, e: float, nchild: int = 8,
               idx: np.ndarray | None = None, threads: int = 0) -> np.ndarray:
    """Reference astro2 (nchild 8) / astro (nchild 4) accelerations.  With idx,
    only those bodies (the tree is built from all of them)."""
    lib = load()
    _, ACC = _entity_dtype()
    state = _ent(state)
    if idx is None:
        out = np.zeros(len(state), dtype=ACC)
        st = lib.oracle_barnes_hut(nchild, state.ctypes.data, len(state), theta, e, None, 0,
                                   out.ctypes.data, threads)
    else:
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        out = np.zeros(len(idx), dtype=ACC)
        st = lib.oracle_barnes_hut(nchild, state.ctypes.data, len(state), theta, e,
                                   idx.ctypes.data, len(idx), out.ctypes.data, threads)
    if st != 0:
        raise RuntimeError(f"reference tree panics (status {st})")
    return out


INTEGRATORS = {"verlet": 0, "euler": 1, "rk4": 2}


def run_pipeline(state: np.ndarray, element: str, steps: int, dt: float, e: float,
                 theta: float = 1.0, threads: int = 0, integrator: str = "verlet") -> np.ndarray:
    """pipeline.rs loop with one gravity element + one integrator (verlet,
    euler or rk4); returns the final state."""
    lib = load()
    s = np.array(_ent(state), copy=True)
    code = {"simple_astro": 0, "astro2": 1, "astro": 2}[element]
    st = lib.oracle_run_pipeline_with(s.ctypes.data, len(s), code, INTEGRATORS[integrator],
                                      theta, e, dt, steps, threads)
    if st != 0:
        raise RuntimeError(f"reference tree panics (status {st})")
    return s


def euler_step(entities: np.ndarray, acc: np.ndarray, dt: float) -> np.ndarray:
    """euler.rs:17-49 given the accelerations acc_fn produced."""
    lib = load()
    entities, acc = _ent(entities), _acc(acc)
    out = np.empty_like(entities)
    lib.oracle_euler_step(entities.ctypes.data, out.ctypes.data, len(entities), acc.ctypes.data,
                          dt)
    return out


ACC_FN = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p)


def rk4_step(entities: np.ndarray, acc_fn, dt: float) -> np.ndarray:
    """rk4.rs:24-178 with a Python acc_fn(state, acc) that adds into acc."""
    from physim_gb300.entity import ACCELERATION, ENTITY
    lib = load()
    entities = _ent(entities)
    out = np.empty_like(entities)

    def cb(_user, sp, n, ap):
        st = np.ctypeslib.as_array(C.cast(sp, C.POINTER(C.c_uint8)), (n * ENTITY.itemsize,))
        ac = np.ctypeslib.as_array(C.cast(ap, C.POINTER(C.c_uint8)), (n * 24,))
        acc_fn(st.view(ENTITY), ac.view(ACCELERATION))

    fn = ACC_FN(cb)
    if lib.oracle_rk4_step(entities.ctypes.data, out.ctypes.data, len(entities),
                           C.cast(fn, C.c_void_p), None, dt) != 0:
        raise MemoryError("rk4 oracle: out of memory")
    return out


class Verlet:
    """verlet.rs restated (previous_state kept between calls)."""

    def __init__(self):
        self.lib = load()
        self.h = self.lib.oracle_verlet_new()

    def step(self, entities: np.ndarray, acc: np.ndarray, dt: float) -> np.ndarray:
        entities, acc = _ent(entities), _acc(acc)
        out = np.empty_like(entities)
        self.lib.oracle_verlet_step(self.h, entities.ctypes.data, out.ctypes.data, len(entities),
                                    acc.ctypes.data, dt)
        return out

    def __del__(self):
        try:
            self.lib.oracle_verlet_free(self.h)
        except Exception:
            pass


class Tree:
    """The reference pointer octree (nchild 8) / quadtree (nchild 4)."""

    def __init__(self, nchild: int, centre=(0.0, 0.0, 0.0), extent: float = 1.0):
        self.lib = load()
        c = (C.c_double * 3)(*centre)
        self.h = self.lib.oracle_tree_new(nchild, c, extent)
        if not self.h:
            raise ValueError("bad tree arguments")

    def push(self, entity) -> int:
        ENTITY, _ = _entity_dtype()
        e = np.array(entity, dtype=ENTITY)
        return self.lib.oracle_tree_push(self.h, e.ctypes.data)

    def leaves(self, loc, theta: float, with_entities: bool = False):
        ENTITY, _ = _entity_dtype()
        c = (C.c_double * 3)(*loc)
        n = self.lib.oracle_tree_leaves(self.h, c, theta, None, 0)
        if not with_entities:
            return n
        out = np.zeros(n, dtype=ENTITY)
        self.lib.oracle_tree_leaves(self.h, c, theta, out.ctypes.data, n)
        return out

    def node_count(self) -> int:
        return self.lib.oracle_tree_node_count(self.h)

    def __del__(self):
        try:
            self.lib.oracle_tree_free(self.h)
        except Exception:
            pass


def bh_model(state: np.ndarray, nchild: int = 8, leaf: int = 16) -> dict:
    """The CPU model of the GPU tree build (bh_model.c): keys, sort order and
    the level-by-level tree, for bit-exact comparison with the GPU."""
    lib = load()
    state = _ent(state)
    n = len(state)
    cap = 4 * max(n, 64) + 64 * 31
    keys = np.zeros(n, np.uint64)
    order = np.zeros(n, np.uint32)
    nb = np.zeros(cap, np.int32)
    nc = np.zeros(cap, np.int32)
    ch = np.zeros(cap, np.int32)
    nn = np.zeros(cap, np.uint8)
    lvl = np.zeros(cap, np.uint8)
    cen = np.zeros(4 * cap, np.float64)
    total = lib.bh_model_build(state.ctypes.data, n, nchild, leaf, keys.ctypes.data,
                               order.ctypes.data, nb.ctypes.data, nc.ctypes.data, ch.ctypes.data,
                               nn.ctypes.data, lvl.ctypes.data, cen.ctypes.data, cap)
    if total < 0:
        raise RuntimeError("model tree capacity exceeded")
    m = int(total)
    cen = cen.reshape(4, cap)[:, :m]
    return {"keys": keys, "order": order, "begin": nb[:m], "count": nc[:m], "child": ch[:m],
            "nchild": nn[:m], "level": lvl[:m], "centre": cen,
            "extent": lib.bh_model_extent(state.ctypes.data, n)}


def bh_model_accel(state: np.ndarray, theta: float, e: float, idx: np.ndarray, nchild: int = 8,
                   leaf: int = 16, quad: bool = False, com_theta: float = 0.0) -> np.ndarray:
    """f64 model of the GPU traversal's accuracy options (per-body rule): the
    reference's opening rule, optionally the centre-of-mass guard and the
    quadrupole term, over the model tree.  Returns (len(idx), 3)."""
    lib = load()
    state = _ent(state)
    idx = np.ascontiguousarray(idx, dtype=np.int64)
    out = np.zeros((len(idx), 3))
    if lib.bh_model_accel(state.ctypes.data, len(state), nchild, leaf, theta, e,
                          1 if quad else 0, com_theta, idx.ctypes.data, len(idx),
                          out.ctypes.data) != 0:
        raise MemoryError("bh_model_accel: out of memory")
    return out


def cube(props: dict) -> np.ndarray:
    """The `cube` initialiser restated (same variates as the GPU generator)."""
    from physim_gb300.initialisers import CUBE_DEFAULTS
    q = {**CUBE_DEFAULTS, **props}
    ENTITY, _ = _entity_dtype()
    out = np.zeros(int(q["n"]), dtype=ENTITY)
    load().oracle_cube(int(q["seed"]), float(q["spin"]), float(q["size"]), float(q["mass"]),
                       (C.c_double * 3)(*q["centre"]), int(q["id"]), len(out), out.ctypes.data)
    return out


def plummer(props: dict) -> np.ndarray:
    """The `plummer` initialiser restated (same variates as the GPU generator)."""
    from physim_gb300.initialisers import PLUMMER_DEFAULTS
    q = {**PLUMMER_DEFAULTS, **props}
    ENTITY, _ = _entity_dtype()
    out = np.zeros(int(q["n"]), dtype=ENTITY)
    load().oracle_plummer(int(q["seed"]), float(q["mass"]), float(q["a"]), float(q["spin"]),
                          (C.c_double * 3)(*q["centre"]), (C.c_double * 3)(*q["v"]),
                          int(q["id"]), len(out), out.ctypes.data)
    return out
