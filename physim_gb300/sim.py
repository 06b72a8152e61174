"""Device-resident simulations (physim_gpu_sim_* in include/physim_gb300.h)."""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from ._lib import (GRAVITY_ASTRO, GRAVITY_ASTRO2, GRAVITY_SIMPLE_ASTRO, INTEGRATOR_EULER,
                   INTEGRATOR_RK4, INTEGRATOR_VERLET, TRAVERSAL_EXACT, TRAVERSAL_WARP,
                   PhysimSimConfig, check, lib)
from .entity import ACCELERATION, ENTITY, as_entities

GRAVITY = {"simple_astro": GRAVITY_SIMPLE_ASTRO, "astro2": GRAVITY_ASTRO2, "astro": GRAVITY_ASTRO}
TRAVERSAL = {"exact": TRAVERSAL_EXACT, "warp": TRAVERSAL_WARP}
INTEGRATOR = {"verlet": INTEGRATOR_VERLET, "euler": INTEGRATOR_EULER, "rk4": INTEGRATOR_RK4}


@dataclass
class SimConfig:
    gravity: str = "simple_astro"
    theta: float = 1.0
    e: float = 1.0
    dt: float = 1e-6
    leaf_size: int = 1
    traversal: str = "exact"
    compensated: bool = True
    device: int = 0
    stream: int | None = None  # a cudaStream_t (e.g. torch.cuda.Stream().cuda_stream)
    integrator: str = "verlet"  # verlet, euler or rk4 (integrators/src/)
    # accuracy options of astro/astro2 beyond the reference (off by default)
    quadrupole: bool = False  # add the cells' quadrupole moments
    com_theta: float = 0.0    # > 0: also require b_max < com_theta |x - c| to accept a cell

    def to_c(self) -> PhysimSimConfig:
        c = PhysimSimConfig()
        lib.physim_gpu_sim_config_default(C.byref(c))
        c.gravity = GRAVITY[self.gravity]
        c.theta = self.theta
        c.e = self.e
        c.dt = self.dt
        c.leaf_size = self.leaf_size
        c.traversal = TRAVERSAL[self.traversal]
        c.compensated = 1 if self.compensated else 0
        c.device = self.device
        c.stream = self.stream or None
        c.integrator = INTEGRATOR[self.integrator]
        c.multipole = 1 if self.quadrupole else 0
        c.com_theta = self.com_theta
        return c


class Simulation:
    """A simulation whose state stays on the GPU between steps."""

    def __init__(self, state: np.ndarray, config: SimConfig):
        state = as_entities(state)
        self.n = len(state)
        self.config = config
        h = C.c_void_p()
        cfg = config.to_c()
        check(lib.physim_gpu_sim_create(C.byref(cfg), self.n, C.byref(h)),
              "physim_gpu_sim_create")
        self.handle = h
        self.upload(state)

    @classmethod
    def generated(cls, kind: str, props: dict, config: SimConfig) -> "Simulation":
        """A simulation whose bodies are generated on the device by the `cube`
        or `plummer` initialiser (physim_gb300.initialisers) -- no host-side
        generation or upload."""
        from . import initialisers
        n, p = (initialisers.cube_params(props) if kind == "cube"
                else initialisers.plummer_params(props))
        self = cls.__new__(cls)
        self.n = n
        self.config = config
        h = C.c_void_p()
        cfg = config.to_c()
        check(lib.physim_gpu_sim_create(C.byref(cfg), n, C.byref(h)), "physim_gpu_sim_create")
        self.handle = h
        fn = lib.physim_gpu_sim_init_cube if kind == "cube" else lib.physim_gpu_sim_init_plummer
        check(fn(self.handle, C.byref(p)), "physim_gpu_sim_init_" + kind)
        return self

    def run(self, steps: int, sink=None) -> None:
        """Advances `steps` steps, handing the state to `sink.render` before
        the first step and after every sink.print_n-th step (the states a
        physim renderer receives, pipeline.rs:130-181)."""
        if sink is None:
            self.step(steps)
            return
        sink.render(self.download())
        every = max(1, int(sink.print_n))
        done = 0
        while done < steps:
            k = min(every, steps - done)
            self.step(k)
            done += k
            if done % every == 0:
                sink.render(self.download(), iteration=done)

    def upload(self, state: np.ndarray) -> None:
        state = as_entities(state)
        check(lib.physim_gpu_sim_upload(self.handle, state.ctypes.data, len(state)),
              "physim_gpu_sim_upload")

    def step(self, steps: int = 1) -> None:
        check(lib.physim_gpu_sim_step(self.handle, steps), "physim_gpu_sim_step")

    def synchronize(self) -> None:
        check(lib.physim_gpu_sim_synchronize(self.handle), "physim_gpu_sim_synchronize")

    def download(self) -> np.ndarray:
        out = np.empty(self.n, dtype=ENTITY)
        check(lib.physim_gpu_sim_download(self.handle, out.ctypes.data, self.n),
              "physim_gpu_sim_download")
        return out

    def accelerations(self) -> np.ndarray:
        out = np.empty(self.n, dtype=ACCELERATION)
        check(lib.physim_gpu_sim_accelerations(self.handle, out.ctypes.data, self.n),
              "physim_gpu_sim_accelerations")
        return out

    def accelerations_f64(self, idx) -> np.ndarray:
        """The reference's direct-sum accelerations in f64 of the bodies `idx`
        of the current state (an accuracy reference for every element)."""
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        out = np.empty(len(idx), dtype=ACCELERATION)
        check(lib.physim_gpu_sim_accelerations_f64(self.handle, idx.ctypes.data, len(idx),
                                                   out.ctypes.data),
              "physim_gpu_sim_accelerations_f64")
        return out

    def tree_snapshot(self) -> dict:
        """Keys, sort order and tree of the current state (astro/astro2 only)."""
        from ._lib import PhysimTreeSnapshot
        cap = 4 * max(self.n, 64) + 64 * 31
        keys = np.zeros(self.n, np.uint64)
        order = np.zeros(self.n, np.uint32)
        nb, nc, ch = (np.zeros(cap, np.int32) for _ in range(3))
        nn, lvl = np.zeros(cap, np.uint8), np.zeros(cap, np.uint8)
        cen = np.zeros(4 * cap, np.float64)
        com = np.zeros(4 * cap, np.float32)
        quad = np.zeros(8 * cap, np.float32)
        s = PhysimTreeSnapshot()
        s.cap_nodes = cap
        for name, arr in (("keys", keys), ("order", order), ("node_begin", nb),
                          ("node_count", nc), ("node_child", ch), ("node_nchild", nn),
                          ("node_level", lvl), ("node_centre", cen), ("node_com", com),
                          ("node_quad", quad)):
            setattr(s, name, arr.ctypes.data)
        check(lib.physim_gpu_sim_tree_snapshot(self.handle, C.byref(s)),
              "physim_gpu_sim_tree_snapshot")
        m = min(s.n_nodes, cap)
        return {"keys": keys, "order": order, "begin": nb[:m], "count": nc[:m], "child": ch[:m],
                "nchild": nn[:m], "level": lvl[:m], "centre": cen[:4 * m].reshape(4, m),
                "com": com[:4 * m].reshape(m, 4), "n_nodes": int(s.n_nodes),
                "quad": np.concatenate([quad[:4 * m].reshape(m, 4),
                                        quad[4 * m:8 * m].reshape(m, 4)], axis=1),
                "extent": s.extent, "flags": int(s.flags)}

    def diagnostics(self, potential: bool = False) -> dict:
        """f64 mass, centre of mass, momentum, kinetic and (optionally) potential
        energy of the current state."""
        from ._lib import PhysimDiagnostics
        d = PhysimDiagnostics()
        check(lib.physim_gpu_sim_diagnostics(self.handle, C.byref(d), 1 if potential else 0),
              "physim_gpu_sim_diagnostics")
        return {"mass": d.mass, "centre_of_mass": list(d.centre_of_mass),
                "momentum": list(d.momentum), "kinetic": d.kinetic,
                "potential": d.potential if potential else None,
                "energy": d.energy if potential else None}

    def bh_stats(self) -> dict:
        """Node visits and pair interactions of the most recent traversal."""
        v, i, t = C.c_uint64(), C.c_uint64(), C.c_double()
        check(lib.physim_gpu_sim_bh_stats(self.handle, C.byref(v), C.byref(i), C.byref(t)),
              "physim_gpu_sim_bh_stats")
        return {"node_visits": v.value, "interactions": i.value, "traversal_ms": t.value}

    def autotune(self) -> dict:
        """Times the candidate pair-kernel plans (simple_astro) and keeps the
        fastest; returns the chosen plan."""
        from ._lib import PhysimDirectTuning
        t = PhysimDirectTuning()
        check(lib.physim_gpu_sim_autotune(self.handle, C.byref(t)), "physim_gpu_sim_autotune")
        return {"block": t.block, "ipt": t.ipt, "splits": t.splits, "candidates": t.candidates,
                "symmetric": bool(t.symmetric), "tiles": t.tiles, "force_ms": t.force_ms}

    def plan(self) -> dict:
        """The current pair-kernel plan (simple_astro)."""
        from ._lib import PhysimDirectTuning
        t = PhysimDirectTuning()
        check(lib.physim_gpu_sim_plan(self.handle, C.byref(t)), "physim_gpu_sim_plan")
        return {"block": t.block, "ipt": t.ipt, "splits": t.splits,
                "symmetric": bool(t.symmetric), "tiles": t.tiles}

    def set_plan(self, symmetric: bool = False, block: int = 256, ipt: int = 4,
                 splits: int = 1) -> None:
        """Fixes the pair-kernel plan (simple_astro): every unordered pair once
        (`symmetric`), or a one-pair kernel of `block` threads with `ipt`
        bodies per thread and `splits` j-range splits."""
        from ._lib import PhysimDirectTuning
        t = PhysimDirectTuning()
        t.symmetric, t.block, t.ipt, t.splits = int(symmetric), block, ipt, splits
        check(lib.physim_gpu_sim_set_plan(self.handle, C.byref(t)), "physim_gpu_sim_set_plan")

    def set_profiling(self, enable: bool = True) -> None:
        check(lib.physim_gpu_sim_set_profiling(self.handle, 1 if enable else 0),
              "physim_gpu_sim_set_profiling")

    def last_step_ms(self) -> tuple[float, float]:
        """(gravity kernels, integrator) device milliseconds of the last step."""
        g, i = C.c_double(), C.c_double()
        check(lib.physim_gpu_sim_last_step_ms(self.handle, C.byref(g), C.byref(i)),
              "physim_gpu_sim_last_step_ms")
        return g.value, i.value

    def last_pair_ms(self) -> float:
        """Device milliseconds of the last step's pair kernel (simple_astro)."""
        v = C.c_double()
        check(lib.physim_gpu_sim_last_pair_ms(self.handle, C.byref(v)),
              "physim_gpu_sim_last_pair_ms")
        return v.value

    @property
    def stream(self) -> int:
        return lib.physim_gpu_sim_stream(self.handle) or 0

    @property
    def launches_per_step(self) -> int:
        return lib.physim_gpu_sim_launches_per_step(self.handle)

    def close(self) -> None:
        if self.handle:
            lib.physim_gpu_sim_destroy(self.handle)
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
