"""The Rust plugin crate (rust/physim_gb300_plugin) cannot be built here (no
cargo), so its contract with the library is checked as text: every function
its `extern "C"` block declares exists in include/physim_gb300.h with the
same argument and return types, is exported by libphysim_gb300.so, and the
`#[repr(C)]` Diagnostics struct has PhysimDiagnostics' fields in order; the
crate registers physim's element names (integrators/src/lib.rs:3,
debug/src/energysink.rs:14) and makes the ABI string as astro/build.rs:3-9."""
from __future__ import annotations

import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
CRATE = ROOT / "rust" / "physim_gb300_plugin"
HEADER = ROOT / "include" / "physim_gb300.h"

# opaque handle types of the header: the crate passes them as *mut c_void
OPAQUE = {"PhysimSim", "PhysimEnsemble", "PhysimVerlet", "PhysimIntegrator", "PhysimEnergy"}

RUST_TYPES = {
    "c_int": "int", "i32": "int32", "u32": "uint32", "u64": "uint64", "usize": "size",
    "f64": "double", "f32": "float", "AccFn": "PhysimAccFn", "*const c_char": "const char*",
    "*mut c_void": "void*", "*mut *mut c_void": "void**", "*const Entity": "const Entity*",
    "*mut Entity": "Entity*", "*const Acceleration": "const Acceleration*",
    "*mut Acceleration": "Acceleration*", "*mut Diagnostics": "PhysimDiagnostics*",
}
C_TYPES = {"int": "int", "int32_t": "int32", "uint32_t": "uint32", "uint64_t": "uint64",
           "size_t": "size", "double": "double", "float": "float"}


def rust_extern_fns(src: str) -> dict[str, tuple[list[str], str | None]]:
    block = src[src.index('unsafe extern "C" {'):]
    block = block[:block.index("\n}\n")]
    out = {}
    for m in re.finditer(r"pub fn (\w+)\((.*?)\)\s*(?:->\s*([^;]+))?;", block, re.S):
        args = [a.strip() for a in m.group(2).replace("\n", " ").split(",") if a.strip()]
        types = [RUST_TYPES[a.split(":", 1)[1].strip()] for a in args]
        ret = RUST_TYPES[m.group(3).strip()] if m.group(3) else None
        out[m.group(1)] = (types, ret)
    return out


def _c_type(t: str) -> str:
    t = " ".join(t.replace("*", " * ").split())
    stars = t.count("*")
    base = t.replace("*", "").strip()
    const = base.startswith("const ")
    base = base.replace("const ", "").strip()
    if base in OPAQUE:
        return "void" + "*" * stars
    if stars == 0:
        return C_TYPES.get(base, base)
    return ("const " if const else "") + base + "*" * stars


def c_decl(header: str, name: str) -> tuple[list[str], str | None]:
    m = re.search(r"([\w\s\*]+?)\b" + name + r"\s*\(([^)]*)\)\s*;", header)
    assert m, f"{name} is not declared in include/physim_gb300.h"
    ret = _c_type(m.group(1).split(";")[-1].split("*/")[-1].strip())
    params = []
    for p in m.group(2).split(","):
        p = " ".join(p.split())
        if not p or p == "void":
            continue
        p = re.sub(r"\s*\b\w+$", "", p) if not p.endswith("*") else p  # drop the name
        params.append(_c_type(p))
    return params, (None if ret == "void" else ret)


def test_extern_block_matches_header():
    src = (CRATE / "src" / "ffi.rs").read_text()
    header = HEADER.read_text()
    fns = rust_extern_fns(src)
    assert {"physim_gpu_integrator_integrate", "physim_gpu_energy_compute",
            "physim_gpu_last_error"} <= set(fns)
    for name, (args, ret) in fns.items():
        c_args, c_ret = c_decl(header, name)
        assert args == c_args, (name, args, c_args)
        assert ret == c_ret, (name, ret, c_ret)


def test_extern_block_symbols_are_exported():
    from test_abi import exported_symbols

    import physim_gb300
    exported = exported_symbols(physim_gb300.LIB_PATH)
    for name in rust_extern_fns((CRATE / "src" / "ffi.rs").read_text()):
        assert name in exported, name


def test_diagnostics_struct_layout():
    src = (CRATE / "src" / "ffi.rs").read_text()
    body = re.search(r"pub struct Diagnostics \{(.*?)\}", src, re.S).group(1)
    rust = [(n, t.strip().rstrip(",")) for n, t in re.findall(r"pub (\w+): ([^\n]+)", body)]
    header = HEADER.read_text()
    cbody = re.search(r"typedef struct PhysimDiagnostics \{(.*?)\} PhysimDiagnostics;", header,
                      re.S).group(1)
    cfields = []
    for m in re.finditer(r"double\s+(\w+)(\[3\])?;", re.sub(r"/\*.*?\*/", "", cbody, flags=re.S)):
        cfields.append((m.group(1), "[f64; 3]" if m.group(2) else "f64"))
    assert rust == cfields
    from physim_gb300._lib import PhysimDiagnostics
    assert [f for f, _ in PhysimDiagnostics._fields_] == [n for n, _ in cfields]


def test_integrator_kinds_match_header():
    src = (CRATE / "src" / "ffi.rs").read_text()
    header = HEADER.read_text()
    for kind in ("VERLET", "EULER", "RK4"):
        rust = int(re.search(rf"INTEGRATOR_{kind}: u32 = (\d+);", src).group(1))
        c = int(re.search(rf"PHYSIM_INTEGRATOR_{kind}\s*=\s*(\d+)", header).group(1))
        assert rust == c, kind


def test_element_names_and_abi_string():
    lib = (CRATE / "src" / "lib.rs").read_text()
    assert 'register_plugin!("verlet", "euler", "rk4", "energysink");' in lib
    names = re.findall(r'#\[(?:integrator|render)_element\(name = "(\w+)"',
                       (CRATE / "src" / "integrators.rs").read_text() +
                       (CRATE / "src" / "energysink.rs").read_text())
    assert sorted(names) == ["energysink", "euler", "rk4", "verlet"]
    build = (CRATE / "build.rs").read_text()
    assert 'cargo:rustc-env=ABI_INFO=rustc:{}|target:{}' in build
    assert "cargo:rustc-link-lib=dylib=physim_gb300" in build
    manifest = (CRATE / "Cargo.toml").read_text()
    assert 'crate-type = ["dylib"]' in manifest and "rustc_version" in manifest
