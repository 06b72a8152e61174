"""Batched ensembles of independent direct-sum simulations (physim_gpu_ensemble_*)."""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from ._lib import PhysimEnsembleTuning, check, lib
from .entity import ENTITY, as_entities
from .sim import SimConfig

UNLIMITED = (1 << 64) - 1


class Ensemble:
    """Members of uneven size advanced together by one persistent pair kernel
    per step (a work queue over all members), replayed from a CUDA graph."""

    def __init__(self, states: Sequence[np.ndarray], config: SimConfig,
                 steps: Sequence[int] | None = None, params: Sequence[tuple] | None = None):
        self.sizes = [len(s) for s in states]
        sizes = (C.c_size_t * len(self.sizes))(*self.sizes)
        h = C.c_void_p()
        cfg = config.to_c()
        check(lib.physim_gpu_ensemble_create(C.byref(cfg), sizes, len(self.sizes), C.byref(h)),
              "physim_gpu_ensemble_create")
        self.handle = h
        self.config = config
        for k, s in enumerate(states):
            self.upload(k, s)
            e, dt = params[k] if params is not None else (config.e, config.dt)
            budget = UNLIMITED if steps is None else int(steps[k])
            self.set_member(k, e, dt, budget)

    @classmethod
    def slots(cls, capacities: Sequence[int], config: SimConfig) -> "Ensemble":
        """An ensemble of empty member slots (each able to hold up to its
        capacity of bodies), for continuous batching: resize_member + upload +
        set_member put a job in a slot."""
        self = cls.__new__(cls)
        self.sizes = [int(c) for c in capacities]
        sizes = (C.c_size_t * len(self.sizes))(*self.sizes)
        h = C.c_void_p()
        cfg = config.to_c()
        check(lib.physim_gpu_ensemble_create(C.byref(cfg), sizes, len(self.sizes), C.byref(h)),
              "physim_gpu_ensemble_create")
        self.handle = h
        self.config = config
        for k in range(len(self.sizes)):
            self.resize_member(k, 0)
        return self

    def upload(self, index: int, state: np.ndarray) -> None:
        state = as_entities(state)
        check(lib.physim_gpu_ensemble_upload(self.handle, index, state.ctypes.data, len(state)),
              "physim_gpu_ensemble_upload")

    def resize_member(self, index: int, n: int) -> None:
        """Reuses member `index`'s slot for n bodies (at most its original
        count); upload and set_member before it steps again."""
        check(lib.physim_gpu_ensemble_resize_member(self.handle, index, n),
              "physim_gpu_ensemble_resize_member")
        self.sizes[index] = n

    def set_member(self, index: int, e: float, dt: float, steps_remaining: int = UNLIMITED) -> None:
        check(lib.physim_gpu_ensemble_set_member(self.handle, index, e, dt, steps_remaining),
              "physim_gpu_ensemble_set_member")

    def autotune(self) -> dict:
        t = PhysimEnsembleTuning()
        check(lib.physim_gpu_ensemble_autotune(self.handle, C.byref(t)),
              "physim_gpu_ensemble_autotune")
        return {"block": t.block, "ipt": t.ipt, "chunk_bodies": t.chunk_bodies,
                "candidates": t.candidates, "symmetric_from": t.symmetric_from,
                "force_ms": t.force_ms}

    def step(self, steps: int = 1) -> None:
        check(lib.physim_gpu_ensemble_step(self.handle, steps), "physim_gpu_ensemble_step")

    def synchronize(self) -> None:
        check(lib.physim_gpu_ensemble_synchronize(self.handle), "physim_gpu_ensemble_synchronize")

    def download(self, index: int) -> np.ndarray:
        out = np.empty(self.sizes[index], dtype=ENTITY)
        check(lib.physim_gpu_ensemble_download(self.handle, index, out.ctypes.data, len(out)),
              "physim_gpu_ensemble_download")
        return out

    def progress(self) -> tuple[np.ndarray, np.ndarray]:
        done = np.zeros(len(self.sizes), np.uint64)
        rem = np.zeros(len(self.sizes), np.uint64)
        check(lib.physim_gpu_ensemble_progress(self.handle, done.ctypes.data, rem.ctypes.data),
              "physim_gpu_ensemble_progress")
        return done, rem

    @property
    def stream(self) -> int:
        return lib.physim_gpu_ensemble_stream(self.handle) or 0

    @property
    def launches_per_step(self) -> int:
        return lib.physim_gpu_ensemble_launches_per_step(self.handle)

    def close(self) -> None:
        if self.handle:
            lib.physim_gpu_ensemble_destroy(self.handle)
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
