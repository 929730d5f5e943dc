"""Builds libcellsim.so in-tree with nvcc for sm_103a.

Translation units are compiled in parallel; the shared library links the
CUDA runtime statically, so the only run-time dependency is the driver.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libcellsim.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["model.cpp", "abi.cpp", "device_ref.cu", "device_prod.cu", "device_stream.cu", "device_resident.cu"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: libcellsim needs the CUDA toolkit to build")


def _compile(src: str, nvcc: str, extra: list[str]) -> Path:
    obj = BUILD / (src + ".o")
    path = CSRC / src
    common = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-lineinfo"] + extra
    if src.endswith(".cu"):
        cmd = [nvcc, *ARCH, *common, "--expt-relaxed-constexpr", "-Xptxas", "-v", "-c", str(path), "-o", str(obj)]
    else:
        cmd = [nvcc, "-x", "c++", *common, "-c", str(path), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    (BUILD / (src + ".log")).write_text(res.stdout + res.stderr)
    if res.returncode != 0:
        raise RuntimeError(f"compiling {src} failed:\n{res.stderr[-6000:]}")
    return obj


def _stale() -> bool:
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = list(CSRC.glob("*")) + [PKG.parent / "include" / "cellsim.h", Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.exists())


def build(force: bool = False, extra: list[str] | None = None) -> Path:
    """Compile every translation unit for sm_103a and link libcellsim.so."""
    if not force and not _stale():
        return LIB
    nvcc = _nvcc()
    BUILD.mkdir(exist_ok=True)
    extra = list(extra or [])
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, extra), SOURCES))
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-cudart", "static"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"linking libcellsim.so failed:\n{res.stderr[-6000:]}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
