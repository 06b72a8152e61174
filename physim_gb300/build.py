"""Builds libphysim_gb300.so (CUDA, sm_103a) in-tree with nvcc.

The library is compiled from physim_gb300/csrc into physim_gb300/_lib/.
Translation units are compiled in parallel; the link uses nvcc so the CUDA
runtime is linked statically and the plugin loads into physim without any
other CUDA library on its search path.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_lib"
OBJ_DIR = ROOT / "_build" / "physim_gb300"
LIB_NAME = "libphysim_gb300.so"
LIB_PATH = OUT_DIR / LIB_NAME

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wextra", "-Wno-unused-parameter"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build physim_gb300")
    return cand


def _cuda_include() -> str:
    return str(Path(_nvcc()).resolve().parent.parent / "include")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(src: Path, headers: list[Path]) -> Path:
    obj = OBJ_DIR / (src.name + ".o")
    if not _stale(obj, [src, *headers]):
        return obj
    if src.suffix == ".cu":
        cmd = [_nvcc(), *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", "-c", str(src), "-o",
               str(obj)]
    else:
        cmd = [os.environ.get("CXX", "g++"), *CXX_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}",
               f"-I{_cuda_include()}", "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def build(force: bool = False, jobs: int | None = None) -> Path:
    """Compiles and links the library; returns its path."""
    OBJ_DIR.mkdir(parents=True, exist_ok=True)
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    srcs = sources()
    headers = sorted(CSRC.glob("*.h")) + sorted(CSRC.glob("*.cuh")) + sorted(INCLUDE.glob("*.h"))
    headers.append(CSRC / "exports.map")
    if force:
        for p in OBJ_DIR.glob("*.o"):
            p.unlink()
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, headers), srcs))
    if force or _stale(LIB_PATH, objs):
        tmp = LIB_PATH.with_suffix(".so.tmp")
        cmd = [_nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-ldl",
               "-Xlinker", f"-soname={LIB_NAME}",
               "-Xlinker", f"--version-script={CSRC / 'exports.map'}"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in os.sys.argv))
