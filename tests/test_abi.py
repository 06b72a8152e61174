"""The C ABI: exported symbols, plugin discovery contract, init/JSON handling,
property descriptions, metadata and bus messages.  No GPU calls."""
from __future__ import annotations

import ctypes as C
import json
import re
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
HEADER = ROOT / "include" / "physim_gb300.h"


def header_functions() -> list[str]:
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    text = re.sub(r"typedef\s+(struct|enum)\s*\w*\s*\{.*?\}\s*\w+\s*;", "", text, flags=re.S)
    text = re.sub(r"typedef[^;]*;", "", text, flags=re.S)
    text = re.sub(r"enum\s*\{.*?\}\s*;", "", text, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", text)
    return sorted(set(names))


def exported_symbols(path: Path) -> set[str]:
    out = subprocess.run(["nm", "-D", "--defined-only", str(path)], capture_output=True,
                         text=True, check=True).stdout
    return {ln.split()[-1] for ln in out.splitlines() if " T " in ln}


def test_library_exports_every_declared_function():
    import physim_gb300
    declared = header_functions()
    assert len(declared) >= 40
    exported = exported_symbols(physim_gb300.LIB_PATH)
    missing = [n for n in declared if n not in exported]
    assert not missing, missing
    # nothing beyond the declared C API leaks out of the library
    assert not [s for s in exported if s.startswith("_Z")]


def test_discovery_contract():
    """discover.rs:327-373: ABI string "C" and the element list."""
    from physim_gb300 import lib
    assert lib.get_plugin_abi_info() == b"C"
    assert lib.register_plugin() == b"astro,astro2,simple_astro"


@pytest.mark.parametrize("name", ["astro", "astro2", "simple_astro"])
def test_register_metadata(name):
    from physim_gb300 import register
    meta = register(name)
    assert meta["kind"] == 1  # ElementKind::Transform
    assert meta["name"] == name
    assert meta["plugin"] and meta["version"] and meta["blurb"]


@pytest.mark.parametrize("name", ["astro", "astro2", "simple_astro"])
def test_vtable_matches_exports(name):
    from physim_gb300 import lib
    api = getattr(lib, f"{name}_get_api")().contents
    for field, suffix in (("init", "init"), ("transform", "transform"), ("destroy", "destroy"),
                          ("get_property_descriptions", "get_property_descriptions"),
                          ("recv_message", "recv_message"),
                          ("post_configuration_messages", "post_configuration_messages")):
        fp = C.cast(getattr(api, field), C.c_void_p).value
        sym = C.cast(getattr(lib, f"{name}_{suffix}"), C.c_void_p).value
        assert fp == sym, field
    assert C.sizeof(type(api)) == 48


@pytest.mark.parametrize("raw,ok", [
    (b"{}", True), (b'{"theta": 0.5, "e": 0.01}', True), (b'  {"e": -2}\n', True),
    (b'{"theta": "x", "nested": {"a": [1, 2, {"b": null}]}, "s": "\\u00e9\\n"}', True),
    (b"", False), (b"[]", False), (b"{", False), (b'{"e": 1,}', False), (b"{} x", False),
    (b'{"e": 01}', False), (b'{"e": 1e999}', False), (b"null", False), (b'{"a": tru}', False),
])
@pytest.mark.parametrize("name", ["astro2", "simple_astro"])
def test_init_json(name, raw, ok):
    """transform.rs:72-76 + physim-attribute/src/lib.rs:60-70: init returns
    NULL for text serde_json would reject as a property object."""
    from physim_gb300 import NullElement, TransformElementHandler
    if ok:
        TransformElementHandler(name, raw_json=raw).destroy()
    else:
        with pytest.raises(NullElement):
            TransformElementHandler(name, raw_json=raw)


def test_init_null_config_returns_null():
    from physim_gb300 import lib
    assert not lib.astro2_init(None, 0)


def test_property_descriptions():
    """transformers.rs:182-195,258-263: reference keys and text are kept."""
    from physim_gb300 import TransformElementHandler
    with TransformElementHandler("astro2", {}) as el:
        d = el.get_property_descriptions()
    assert d["theta"].startswith("Barnes-Hut parameter")
    assert d["e"] == "Easing factor. Modify G*Ma*Mb*(r-e)^-2. Default=1.0"
    with TransformElementHandler("simple_astro", {}) as el:
        d = el.get_property_descriptions()
    assert "theta" not in d and "e" in d


def test_descriptions_null_object():
    from physim_gb300 import lib
    from physim_gb300.plugin import HOST_ALLOC
    assert not lib.astro_get_property_descriptions(None, C.cast(HOST_ALLOC, C.c_void_p))


def test_null_objects_are_ignored():
    """A NULL instance is a no-op for every vtable entry (c_plugin/plugin.c)."""
    from physim_gb300 import lib
    lib.simple_astro_transform(None, None, 0, None, 0)
    lib.astro2_destroy(None)
    lib.astro_post_configuration_messages(None)
    lib.astro2_recv_message(None, None)


FAKE_BUS = r"""
#include <stdint.h>
#include <string.h>
typedef struct { int priority; const char *topic; const char *message; uintptr_t sender; int origin; } CMessage;
static char topics[8][64]; static char messages[8][64]; static int origins[8]; static int prios[8];
static void *targets[8]; static int count = 0;
void post_bus_callback(void *target, CMessage m) {
  if (count < 8) { strncpy(topics[count], m.topic, 63); strncpy(messages[count], m.message, 63);
    origins[count] = m.origin; prios[count] = m.priority; targets[count] = target; }
  count++;
}
int bus_count(void) { return count; }
const char *bus_topic(int i) { return topics[i]; }
const char *bus_message(int i) { return messages[i]; }
int bus_origin(int i) { return origins[i]; }
int bus_priority(int i) { return prios[i]; }
void *bus_target(int i) { return targets[i]; }
"""


def test_configuration_message_reaches_bus(tmp_path):
    """post_configuration_messages posts (Low, "energysink", "gravity") with
    origin C through physim's post_bus_callback (transformers.rs:198-203,
    messages.rs:201-226)."""
    src = tmp_path / "fake_bus.c"
    src.write_text(FAKE_BUS)
    so = tmp_path / "libfakebus.so"
    subprocess.run(["gcc", "-shared", "-fPIC", "-o", str(so), str(src)], check=True)
    bus = C.CDLL(str(so), mode=C.RTLD_GLOBAL)
    bus.bus_topic.restype = bus.bus_message.restype = C.c_char_p
    bus.bus_target.restype = C.c_void_p
    from physim_gb300 import TransformElementHandler, lib
    target = C.c_int(7)
    lib.set_callback_target(C.addressof(target))
    with TransformElementHandler("astro2", {"theta": 0.5}) as el:
        el.post_configuration_messages()
    assert bus.bus_count() == 1
    assert bus.bus_topic(0) == b"energysink" and bus.bus_message(0) == b"gravity"
    assert bus.bus_origin(0) == 1  # MessageOrigin::C
    assert bus.bus_priority(0) == 1  # MessagePriority::Low
    assert bus.bus_target(0) == C.addressof(target)


def test_entity_dtype_layout():
    import numpy as np
    from physim_gb300.entity import ACCELERATION, ENTITY, as_entities, entities
    assert ENTITY.itemsize == 80 and ENTITY.fields["id"][1] == 64
    assert ENTITY.fields["fixed"][1] == 72 and ACCELERATION.itemsize == 24
    packed = np.concatenate([entities(2), entities(1)])
    assert as_entities(packed).dtype.itemsize == 80


def test_sim_config_layout():
    from physim_gb300._lib import PhysimSimConfig
    assert C.sizeof(PhysimSimConfig) == 64


def test_host_access_setting():
    """The host-access mode is validated and COPY needs no device query."""
    import physim_gb300 as pg
    from physim_gb300 import lib
    assert lib.physim_gpu_set_host_access(3) != 0  # unknown mode
    try:
        pg.set_host_access("copy")
        assert pg.host_access(0) == "copy"
        assert lib.physim_gpu_host_access(0, None) != 0
    finally:
        pg.set_host_access("auto")


def test_process_wide_plan_knobs_need_no_device():
    """The each-pair-once knobs (slot cap, tile-pair schedule bound), the
    radix look-back limit and the sort's launch mode only store a value:
    callable without a GPU; 0 restores each default (1 for the sort mode)."""
    import physim_gb300 as pg
    from physim_gb300 import lib
    try:
        pg.set_symmetric_cap(1 << 30)
        pg.set_symmetric_pairs_limit(1)
        assert lib.physim_gpu_set_wait_limit(1000) == 0
        assert lib.physim_gpu_set_sort_single_launch(0) == 0
    finally:
        pg.set_symmetric_cap(0)
        pg.set_symmetric_pairs_limit(0)
        assert lib.physim_gpu_set_wait_limit(0) == 0
        assert lib.physim_gpu_set_sort_single_launch(1) == 0
