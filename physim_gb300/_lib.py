"""ctypes binding of libphysim_gb300.so (declarations in include/physim_gb300.h).

`lib` loads the CUDA library on its first use (the first physim_gpu_* or
plugin call), not when the package is imported, so code that only needs the
Entity dtype or the seeded initial conditions (the oracle, the CPU baseline)
never maps the library.  There is no CPU fallback: if the shared library has
not been built, that first call fails with an error that says how to build it.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libphysim_gb300.so"

PHYSIM_OK = 0
PHYSIM_ERR_ARGUMENT = 1
PHYSIM_ERR_CUDA = 2
PHYSIM_ERR_MEMORY = 3
PHYSIM_ERR_TREE = 4
PHYSIM_ERR_TIMEOUT = 5

GRAVITY_SIMPLE_ASTRO = 0
GRAVITY_ASTRO2 = 1
GRAVITY_ASTRO = 2
TRAVERSAL_EXACT = 0
TRAVERSAL_WARP = 1
INTEGRATOR_VERLET = 0
INTEGRATOR_EULER = 1
INTEGRATOR_RK4 = 2
MULTIPOLE_MONOPOLE = 0
MULTIPOLE_QUADRUPOLE = 1
HOST_ACCESS = {"auto": 0, "copy": 1, "direct": 2}


class CMessage(C.Structure):
    _fields_ = [("priority", C.c_int), ("topic", C.c_char_p), ("message", C.c_char_p),
                ("sender_id", C.c_size_t), ("origin", C.c_int)]


class ElementMetaFFI(C.Structure):
    _fields_ = [("kind", C.c_int), ("name", C.c_void_p), ("plugin", C.c_void_p),
                ("version", C.c_void_p), ("license", C.c_void_p), ("author", C.c_void_p),
                ("blurb", C.c_void_p), ("repo", C.c_void_p)]


RustStringAllocFn = C.CFUNCTYPE(C.c_void_p, C.c_char_p)
InitFn = C.CFUNCTYPE(C.c_void_p, C.c_void_p, C.c_size_t)
TransformFn = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p, C.c_size_t)
DestroyFn = C.CFUNCTYPE(None, C.c_void_p)
DescFn = C.CFUNCTYPE(C.c_void_p, C.c_void_p, C.c_void_p)
RecvFn = C.CFUNCTYPE(None, C.c_void_p, C.POINTER(CMessage))
PostFn = C.CFUNCTYPE(None, C.c_void_p)


class TransformElementAPI(C.Structure):
    _fields_ = [("init", InitFn), ("transform", TransformFn), ("destroy", DestroyFn),
                ("get_property_descriptions", DescFn), ("recv_message", RecvFn),
                ("post_configuration_messages", PostFn)]


class PhysimSimConfig(C.Structure):
    _fields_ = [("gravity", C.c_uint32), ("leaf_size", C.c_uint32), ("traversal", C.c_uint32),
                ("compensated", C.c_uint32), ("theta", C.c_double), ("e", C.c_double),
                ("dt", C.c_double), ("stream", C.c_void_p), ("device", C.c_int32),
                ("integrator", C.c_uint32), ("multipole", C.c_uint32),
                ("com_theta", C.c_float)]


# void (*PhysimBusFn)(void *target, const CMessage *message)
BusFn = C.CFUNCTYPE(None, C.c_void_p, C.POINTER(CMessage))

# void (*PhysimAccFn)(void *user, const Entity *state, size_t n, Acceleration *acc)
AccFn = C.CFUNCTYPE(None, C.c_void_p, C.c_void_p, C.c_size_t, C.c_void_p)


class PhysimTreeSnapshot(C.Structure):
    _fields_ = [("cap_nodes", C.c_size_t), ("keys", C.c_void_p), ("order", C.c_void_p),
                ("node_begin", C.c_void_p), ("node_count", C.c_void_p),
                ("node_child", C.c_void_p), ("node_nchild", C.c_void_p),
                ("node_level", C.c_void_p), ("node_centre", C.c_void_p),
                ("node_com", C.c_void_p), ("node_quad", C.c_void_p), ("n_bodies", C.c_size_t),
                ("n_nodes", C.c_size_t),
                ("extent", C.c_double), ("flags", C.c_uint32)]


class PhysimDiagnostics(C.Structure):
    _fields_ = [("mass", C.c_double), ("centre_of_mass", C.c_double * 3),
                ("momentum", C.c_double * 3), ("kinetic", C.c_double), ("potential", C.c_double),
                ("energy", C.c_double)]


class PhysimCubeParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("spin", C.c_double), ("size", C.c_double),
                ("mass", C.c_double), ("centre", C.c_double * 3), ("id", C.c_uint64)]


class PhysimPlummerParams(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("mass", C.c_double), ("a", C.c_double),
                ("spin", C.c_double), ("centre", C.c_double * 3), ("v", C.c_double * 3),
                ("id", C.c_uint64)]


class PhysimDirectTuning(C.Structure):
    _fields_ = [("block", C.c_uint32), ("ipt", C.c_uint32), ("splits", C.c_uint32),
                ("candidates", C.c_uint32), ("symmetric", C.c_uint32), ("tiles", C.c_uint32),
                ("force_ms", C.c_double)]


class PhysimEnsembleTuning(C.Structure):
    _fields_ = [("block", C.c_uint32), ("ipt", C.c_uint32), ("chunk_bodies", C.c_uint32),
                ("candidates", C.c_uint32), ("symmetric_from", C.c_uint32),
                ("reserved", C.c_uint32), ("force_ms", C.c_double)]


ELEMENTS = ("astro", "astro2", "simple_astro")
ELEMENT_SUFFIXES = ("get_api", "register", "init", "transform", "destroy",
                    "get_property_descriptions", "recv_message", "post_configuration_messages")


def _load() -> C.CDLL:
    if not LIB_PATH.exists():
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; "
            "g.build()\"` (requires nvcc); physim_gb300 has no CPU fallback")
    lib = C.CDLL(str(LIB_PATH), mode=os.RTLD_NOW | os.RTLD_LOCAL)
    vp, sz, i32, u32, dbl = C.c_void_p, C.c_size_t, C.c_int32, C.c_uint32, C.c_double
    sig = {
        "get_plugin_abi_info": (C.c_char_p, []),
        "register_plugin": (C.c_char_p, []),
        "set_callback_target": (None, [vp]),
        "physim_gpu_last_error": (C.c_char_p, []),
        "physim_gpu_set_host_access": (C.c_int, [u32]),
        "physim_gpu_host_access": (C.c_int, [i32, C.POINTER(u32)]),
        "physim_gpu_sim_config_default": (None, [C.POINTER(PhysimSimConfig)]),
        "physim_gpu_sim_create": (C.c_int, [C.POINTER(PhysimSimConfig), sz, C.POINTER(vp)]),
        "physim_gpu_sim_upload": (C.c_int, [vp, vp, sz]),
        "physim_gpu_sim_step": (C.c_int, [vp, u32]),
        "physim_gpu_sim_download": (C.c_int, [vp, vp, sz]),
        "physim_gpu_sim_accelerations": (C.c_int, [vp, vp, sz]),
        "physim_gpu_sim_accelerations_f64": (C.c_int, [vp, vp, sz, vp]),
        "physim_gpu_sim_synchronize": (C.c_int, [vp]),
        "physim_gpu_sim_stream": (vp, [vp]),
        "physim_gpu_sim_launches_per_step": (C.c_int, [vp]),
        "physim_gpu_sim_set_profiling": (C.c_int, [vp, C.c_int]),
        "physim_gpu_sim_last_step_ms": (C.c_int, [vp, C.POINTER(dbl), C.POINTER(dbl)]),
        "physim_gpu_sim_last_pair_ms": (C.c_int, [vp, C.POINTER(dbl)]),
        "physim_gpu_sim_destroy": (None, [vp]),
        "physim_gpu_sim_diagnostics": (C.c_int, [vp, C.POINTER(PhysimDiagnostics), C.c_int]),
        "physim_gpu_sim_tree_snapshot": (C.c_int, [vp, C.POINTER(PhysimTreeSnapshot)]),
        "physim_gpu_sim_autotune": (C.c_int, [vp, C.POINTER(PhysimDirectTuning)]),
        "physim_gpu_sim_set_plan": (C.c_int, [vp, C.POINTER(PhysimDirectTuning)]),
        "physim_gpu_sim_plan": (C.c_int, [vp, C.POINTER(PhysimDirectTuning)]),
        "physim_gpu_set_symmetric_cap": (C.c_int, [C.c_uint64]),
        "physim_gpu_set_symmetric_pairs_limit": (C.c_int, [C.c_uint64]),
        "physim_gpu_set_bus_callback": (C.c_int, [BusFn]),
        "physim_gpu_set_wait_limit": (C.c_int, [u32]),
        "physim_gpu_test_stall_sort": (C.c_int, [i32]),
        "physim_gpu_set_sort_single_launch": (C.c_int, [i32]),
        "physim_gpu_energy_create": (C.c_int, [i32, C.POINTER(vp)]),
        "physim_gpu_energy_compute": (C.c_int, [vp, vp, sz, dbl, C.c_int,
                                                C.POINTER(PhysimDiagnostics)]),
        "physim_gpu_energy_destroy": (None, [vp]),
        "physim_gpu_sim_init_cube": (C.c_int, [vp, C.POINTER(PhysimCubeParams)]),
        "physim_gpu_sim_init_plummer": (C.c_int, [vp, C.POINTER(PhysimPlummerParams)]),
        "physim_gpu_generate_cube": (C.c_int, [C.POINTER(PhysimCubeParams), vp, sz, i32]),
        "physim_gpu_generate_plummer": (C.c_int, [C.POINTER(PhysimPlummerParams), vp, sz, i32]),
        "physim_gpu_sim_bh_stats": (C.c_int, [vp, C.POINTER(C.c_uint64),
                                              C.POINTER(C.c_uint64), C.POINTER(dbl)]),
        "physim_gpu_ensemble_create": (C.c_int, [C.POINTER(PhysimSimConfig), vp, sz,
                                                 C.POINTER(vp)]),
        "physim_gpu_ensemble_upload": (C.c_int, [vp, sz, vp, sz]),
        "physim_gpu_ensemble_set_member": (C.c_int, [vp, sz, dbl, dbl, C.c_uint64]),
        "physim_gpu_ensemble_autotune": (C.c_int, [vp, C.POINTER(PhysimEnsembleTuning)]),
        "physim_gpu_ensemble_step": (C.c_int, [vp, u32]),
        "physim_gpu_ensemble_resize_member": (C.c_int, [vp, sz, sz]),
        "physim_gpu_ensemble_download": (C.c_int, [vp, sz, vp, sz]),
        "physim_gpu_ensemble_progress": (C.c_int, [vp, vp, vp]),
        "physim_gpu_ensemble_synchronize": (C.c_int, [vp]),
        "physim_gpu_ensemble_stream": (vp, [vp]),
        "physim_gpu_ensemble_launches_per_step": (C.c_int, [vp]),
        "physim_gpu_ensemble_destroy": (None, [vp]),
        "physim_gpu_verlet_create": (C.c_int, [i32, C.POINTER(vp)]),
        "physim_gpu_verlet_integrate": (C.c_int, [vp, vp, vp, sz, vp, dbl]),
        "physim_gpu_verlet_destroy": (None, [vp]),
        "physim_gpu_integrator_create": (C.c_int, [u32, i32, C.POINTER(vp)]),
        "physim_gpu_integrator_integrate": (C.c_int, [vp, vp, vp, sz, AccFn, vp, dbl]),
        "physim_gpu_integrator_destroy": (None, [vp]),
    }
    for el in ELEMENTS:
        sig[f"{el}_get_api"] = (C.POINTER(TransformElementAPI), [])
        sig[f"{el}_register"] = (ElementMetaFFI, [RustStringAllocFn])
        sig[f"{el}_init"] = (vp, [vp, sz])
        sig[f"{el}_transform"] = (None, [vp, vp, sz, vp, sz])
        sig[f"{el}_destroy"] = (None, [vp])
        sig[f"{el}_get_property_descriptions"] = (vp, [vp, vp])
        sig[f"{el}_recv_message"] = (None, [vp, C.POINTER(CMessage)])
        sig[f"{el}_post_configuration_messages"] = (None, [vp])
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


class _Library:
    """The loaded libphysim_gb300.so, opened on first attribute access."""

    __slots__ = ("_cdll",)

    def __init__(self):
        self._cdll = None

    def load(self) -> C.CDLL:
        if self._cdll is None:
            self._cdll = _load()
        return self._cdll

    @property
    def loaded(self) -> bool:
        return self._cdll is not None

    def __getattr__(self, name):
        return getattr(self.load(), name)


lib = _Library()


class PhysimError(RuntimeError):
    """A physim_gpu_* call returned a non-zero status."""

    def __init__(self, code: int, what: str):
        super().__init__(f"{what} failed with status {code}: {last_error()}")
        self.code = code


def last_error() -> str:
    msg = lib.physim_gpu_last_error()
    return msg.decode(errors="replace") if msg else ""


def check(code: int, what: str) -> None:
    if code != PHYSIM_OK:
        raise PhysimError(code, what)


def set_host_access(mode: str) -> None:
    """How calls taking host arrays move them: "copy" (cudaMemcpyAsync),
    "direct" (kernels read and write the host arrays in place over the
    device's pageable-memory access) or "auto" (direct where supported)."""
    check(lib.physim_gpu_set_host_access(HOST_ACCESS[mode]), "physim_gpu_set_host_access")


def set_symmetric_cap(nbytes: int) -> None:
    """Largest slot buffer the heuristic direct-sum plans give the
    each-pair-once plan (0: a quarter of the device's memory)."""
    check(lib.physim_gpu_set_symmetric_cap(int(nbytes)), "physim_gpu_set_symmetric_cap")


def set_symmetric_pairs_limit(nbytes: int) -> None:
    """Largest slot buffer with which the each-pair-once plan runs one block
    per tile pair; larger problems use the cluster schedule (0: 4 GiB)."""
    check(lib.physim_gpu_set_symmetric_pairs_limit(int(nbytes)),
          "physim_gpu_set_symmetric_pairs_limit")


def host_access(device: int = 0) -> str:
    """The mode calls on `device` use now: "copy" or "direct"."""
    out = C.c_uint32(0)
    check(lib.physim_gpu_host_access(device, C.byref(out)), "physim_gpu_host_access")
    return {1: "copy", 2: "direct"}[out.value]
