"""physim_gb300 -- physim's gravity + integration hot path on GB300 (sm_103a).

The compute lives in libphysim_gb300.so (CUDA kernels behind a C ABI, see
include/physim_gb300.h).  This package is the Python host side: ctypes
bindings, the physim Entity layout as a numpy dtype, a mirror of physim's
transform-element handler and pipeline step, device-resident simulations and
seeded initial conditions.  The CUDA library is loaded on the first call
that needs it (`lib.load()` loads it explicitly); that call fails loudly if
the library is missing: there is no CPU fallback.
"""
from ._lib import (LIB_PATH, PhysimError, host_access, last_error, lib, set_host_access,
                   set_symmetric_cap, set_symmetric_pairs_limit)
from .entity import ACCELERATION, ENTITY, accelerations, entities, entity_new
from .plugin import (GpuIntegrator, GpuVerlet, NullElement, Pipeline, TransformElementHandler,
                     register)
from .sim import SimConfig, Simulation
from .ensemble import Ensemble

__all__ = [
    "LIB_PATH", "PhysimError", "last_error", "lib", "ACCELERATION", "ENTITY", "accelerations",
    "entities", "entity_new", "GpuIntegrator", "GpuVerlet", "NullElement", "Pipeline",
    "TransformElementHandler", "register", "SimConfig", "Simulation", "Ensemble", "host_access",
    "set_host_access", "set_symmetric_cap", "set_symmetric_pairs_limit",
]
