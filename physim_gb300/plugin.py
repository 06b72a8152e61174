"""Host-side mirror of physim's transform-element handler.

`TransformElementHandler` loads an element through the same C ABI that
physim's Rust host uses (physim-core/src/plugin/transform.rs:52-134): it
resolves `{name}_get_api`, calls `init` with the JSON property object, and
calls `transform(obj, state, n, acc, n)` with host Entity / Acceleration
arrays.  `Pipeline` restates the pipeline step that feeds them
(physim-core/src/pipeline.rs:137-141,166-173): zeroed accelerations, every
transform in order, then the integrator.
"""
from __future__ import annotations

import ctypes as C
import json
from typing import Iterable

import numpy as np

from . import _lib
from ._lib import lib, check
from .entity import ACCELERATION, ENTITY, as_accelerations, as_entities

_libc = C.CDLL(None)
_libc.free.argtypes = [C.c_void_p]
_libc.free.restype = None
# physim hands plugins `host_alloc_string` (physim-core/src/plugin/meta.rs:137-155);
# libc's strdup has the same contract and its result is freed with free().
_strdup_addr = C.cast(_libc.strdup, C.c_void_p).value
HOST_ALLOC = _lib.RustStringAllocFn(_strdup_addr)


class NullElement(RuntimeError):
    """init returned NULL (TransformElementLoadError::NullElement, transform.rs:72-76)."""


def _take_string(ptr: int | None) -> str | None:
    if not ptr:
        return None
    s = C.string_at(ptr).decode()
    _libc.free(ptr)
    return s


def register(name: str) -> dict:
    """Calls `{name}_register` with the host allocator and returns the metadata."""
    meta = getattr(lib, f"{name}_register")(HOST_ALLOC)
    out = {"kind": meta.kind}
    for f in ("name", "plugin", "version", "license", "author", "blurb", "repo"):
        out[f] = _take_string(getattr(meta, f))
    return out


class TransformElementHandler:
    """One element instance created through `{name}_get_api()->init`."""

    def __init__(self, name: str, properties: dict | None = None, *, raw_json: bytes | None = None):
        self.name = name
        self.api = getattr(lib, f"{name}_get_api")().contents
        text = raw_json if raw_json is not None else json.dumps(properties or {}).encode()
        buf = C.create_string_buffer(text, len(text))
        self.instance = self.api.init(C.cast(buf, C.c_void_p), len(text))
        if not self.instance:
            raise NullElement(f"{name}: init rejected {text!r}")

    def transform(self, state: np.ndarray, acc: np.ndarray) -> None:
        """acc += this element's accelerations of `state` (in place)."""
        state = as_entities(state)
        if acc.dtype != ACCELERATION or acc.dtype.itemsize != 24:
            raise TypeError("acc must be an ACCELERATION array (updated in place)")
        if not (acc.flags.c_contiguous and acc.flags.writeable):
            raise ValueError("acc must be C-contiguous and writeable")
        self.api.transform(self.instance, state.ctypes.data, len(state), acc.ctypes.data, len(acc))

    def get_property_descriptions(self) -> dict:
        ptr = self.api.get_property_descriptions(self.instance, C.cast(HOST_ALLOC, C.c_void_p))
        s = _take_string(ptr)
        if s is None:
            raise RuntimeError("Unable to load descriptions of properties")
        return json.loads(s)

    def post_configuration_messages(self) -> None:
        self.api.post_configuration_messages(self.instance)

    def recv_message(self, topic: str, message: str, priority: int = 2, sender: int = 0) -> None:
        m = _lib.CMessage(priority, topic.encode(), message.encode(), sender, 0)
        self.api.recv_message(self.instance, C.byref(m))

    def destroy(self) -> None:
        if self.instance:
            self.api.destroy(self.instance)
            self.instance = None

    def __del__(self):
        try:
            self.destroy()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.destroy()


class MessageBus:
    """Host-side mirror of physim's message bus (physim-core/src/messages.rs:
    201-271) for the configuration messages the gravity elements post
    (transformers.rs:107-111,198-203,266-270).  While installed (a `with`
    block) the library hands those messages here through
    physim_gpu_set_bus_callback instead of physim's `post_bus_callback`;
    `deliver` then calls `recv_message(topic, message, priority, sender)` of
    every client, as physim's message thread does (pipeline.rs:113-127)."""

    # the bus pointer handed to set_callback_target (physim passes its
    # Arc<Mutex<MessageBus>>; the library only hands it back); it stays set
    # after the block, as set_callback_target rejects NULL (c_plugin/plugin.c)
    _TARGET = C.c_int(0)

    def __init__(self):
        self.messages: list[tuple[int, str, str, int, int]] = []
        self._pending: list[tuple[int, str, str, int, int]] = []
        self._cb = _lib.BusFn(self._post)

    def _post(self, target, msg) -> None:
        m = msg.contents
        rec = (m.priority, m.topic.decode(), m.message.decode(), m.sender_id or 0, m.origin)
        self.messages.append(rec)
        self._pending.append(rec)

    def deliver(self, clients: Iterable) -> int:
        """Delivers the pending messages, highest priority first; returns how many."""
        pending = sorted(self._pending, key=lambda r: -r[0])
        self._pending.clear()
        for prio, topic, message, sender, _ in pending:
            for c in clients:
                c.recv_message(topic, message, priority=prio, sender=sender)
        return len(pending)

    def __enter__(self):
        lib.set_callback_target(C.addressof(MessageBus._TARGET))
        check(lib.physim_gpu_set_bus_callback(self._cb), "physim_gpu_set_bus_callback")
        return self

    def __exit__(self, *exc):
        lib.physim_gpu_set_bus_callback(_lib.BusFn())


class GpuVerlet:
    """The verlet integrator (integrators/src/verlet.rs) over host arrays, on the GPU."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        check(lib.physim_gpu_verlet_create(device, C.byref(h)), "physim_gpu_verlet_create")
        self.handle = h

    def integrate(self, entities: np.ndarray, acc: np.ndarray, dt: float,
                  out: np.ndarray | None = None) -> np.ndarray:
        """The new state; written into `out` (an ENTITY array of the same
        length, reused across steps as physim's pipeline reuses new_state,
        pipeline.rs:104-173) when given."""
        entities, acc = as_entities(entities), as_accelerations(acc)
        if out is None:
            new_state = np.empty_like(entities)
        else:
            if out.dtype != ENTITY or len(out) != len(entities) or not out.flags.c_contiguous:
                raise ValueError("out must be a C-contiguous ENTITY array of the same length")
            new_state = out
        check(lib.physim_gpu_verlet_integrate(self.handle, entities.ctypes.data,
                                              new_state.ctypes.data, len(entities),
                                              acc.ctypes.data, dt),
              "physim_gpu_verlet_integrate")
        return new_state

    def close(self) -> None:
        if self.handle:
            lib.physim_gpu_verlet_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class GpuIntegrator:
    """The verlet, euler or rk4 integrator element over host arrays, in the
    shape of physim's IntegratorElement::integrate(entities, new_state,
    acc_fn, dt) (physim-core/src/plugin/integrator.rs:5-13): `acc_fn(state,
    acc)` adds into zeroed accelerations and is called once (verlet, euler)
    or four times (rk4); the updates run on the GPU."""

    KINDS = {"verlet": _lib.INTEGRATOR_VERLET, "euler": _lib.INTEGRATOR_EULER,
             "rk4": _lib.INTEGRATOR_RK4}

    def __init__(self, kind: str = "verlet", device: int = 0):
        h = C.c_void_p()
        check(lib.physim_gpu_integrator_create(self.KINDS[kind], device, C.byref(h)),
              "physim_gpu_integrator_create")
        self.kind = kind
        self.handle = h

    def integrate(self, entities: np.ndarray, acc_fn, dt: float) -> np.ndarray:
        entities = as_entities(entities)
        new_state = np.empty_like(entities)
        error: list[BaseException] = []

        def cb(_user, sp, n, ap):
            try:
                st = np.ctypeslib.as_array(C.cast(sp, C.POINTER(C.c_uint8)),
                                           (n * ENTITY.itemsize,)).view(ENTITY)
                ac = np.ctypeslib.as_array(C.cast(ap, C.POINTER(C.c_uint8)),
                                           (n * ACCELERATION.itemsize,)).view(ACCELERATION)
                acc_fn(st, ac)
            except BaseException as exc:  # surfaced after the C call returns
                error.append(exc)

        fn = _lib.AccFn(cb) if len(entities) else _lib.AccFn(lambda *a: None)
        rc = lib.physim_gpu_integrator_integrate(self.handle, entities.ctypes.data,
                                                 new_state.ctypes.data, len(entities), fn, None,
                                                 dt)
        if error:
            raise error[0]
        check(rc, "physim_gpu_integrator_integrate")
        return new_state

    def close(self) -> None:
        if self.handle:
            lib.physim_gpu_integrator_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pipeline:
    """pipeline.rs:137-173 restated: per step the integrator is handed
    `transform_fn` (every transform in order adding into the accelerations
    it is given) and produces the new state.  `run` first lets the elements
    post their configuration messages and delivers them (to the transforms
    and the sinks), then hands each sink the initial state and every new
    state (pipeline.rs:128-181)."""

    def __init__(self, transforms: Iterable[TransformElementHandler],
                 integrator: GpuVerlet | GpuIntegrator, dt: float, sinks: Iterable = ()):
        self.transforms = list(transforms)
        self.integrator = integrator
        self.dt = dt
        self.sinks = list(sinks)

    def transform_fn(self, state: np.ndarray, acc: np.ndarray) -> None:
        for t in self.transforms:
            t.transform(state, acc)

    def step(self, state: np.ndarray) -> np.ndarray:
        if isinstance(self.integrator, GpuIntegrator):
            return self.integrator.integrate(state, self.transform_fn, self.dt)
        acc = np.zeros(len(state), dtype=ACCELERATION)
        self.transform_fn(state, acc)
        return self.integrator.integrate(state, acc, self.dt)

    def configure(self) -> MessageBus:
        """post_configuration_messages of every transform, delivered."""
        with MessageBus() as bus:
            for t in self.transforms:
                t.post_configuration_messages()
        bus.deliver([*self.transforms, *self.sinks])
        return bus

    def run(self, state: np.ndarray, iterations: int) -> np.ndarray:
        self.configure()
        for sink in self.sinks:
            sink.render(state)
        for _ in range(iterations):
            state = self.step(state)
            for sink in self.sinks:
                sink.render(state)
        return state
