"""Builds the in-tree engine library linon_gb300/_lib/liblinon.so.

The library holds the C ABI (include/linon.h): the WGSL front end, the NVRTC
JIT, the BVH builder and the ahead-of-time CUDA kernels for sm_103a.  The
device headers that NVRTC compiles at run time (csrc/device/*) are embedded
into the library as strings, so nothing is read from disk when a field is
compiled.  The CUDA runtime is linked statically (nvcc's default) and the
driver is reached only through it, so the library also loads on a machine
without a GPU.

Usage: python -m linon_gb300.build [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_lib"
LIB = OUT_DIR / "liblinon.so"
BUILD_DIR = PKG / "_build"
CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

DEVICE_HEADERS = ["wgsl_rt.cuh", "march_types.h", "march.cuh"]
CPP_SOURCES = [
    "wgsl/frontend.cpp",
    "runtime/predefined.cpp",
    "runtime/jit.cpp",
    "runtime/bvh.cpp",
    "runtime/api.cpp",
    "runtime/batch.cpp",
    "runtime/serve.cpp",
    "runtime/obj.cpp",
]
CU_SOURCES = ["runtime/kernels.cu", "runtime/noalloc.cu", "runtime/grid.cu", "runtime/selfcheck.cu"]
GENERATED = BUILD_DIR / "embedded_sources.cpp"

CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
            f"-I{CUDA_HOME / 'include'}"]
NVCCFLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off",
             "-fmad=false", f"-I{CUDA_HOME / 'include'}"] + ARCH


def _embed() -> None:
    """Writes the embedded device-source table (raw string literals)."""
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    parts = ['// generated by linon_gb300/build.py from csrc/device/*; do not edit',
             '#include "../csrc/runtime/internal.hpp"', 'namespace linon {',
             'const EmbeddedFile kEmbeddedDeviceSources[] = {']
    for name in DEVICE_HEADERS:
        text = (CSRC / "device" / name).read_text()
        delim = "LINON_EMBED"
        assert f"){delim}\"" not in text
        # split long files into several literals (compiler literal limits)
        chunks = [text[i:i + 16000] for i in range(0, len(text), 16000)] or [""]
        lit = "\n".join(f'R"{delim}({c}){delim}"' for c in chunks)
        parts.append(f'  {{"{name}", {lit}}},')
    parts += ['};', f'const int kEmbeddedDeviceSourceCount = {len(DEVICE_HEADERS)};', '}  // namespace linon', '']
    text = "\n".join(parts)
    if not GENERATED.exists() or GENERATED.read_text() != text:
        GENERATED.write_text(text)


def _digest(paths) -> str:
    h = hashlib.sha256()
    for p in paths:
        h.update(str(p).encode())
        h.update(Path(p).read_bytes())
    h.update(" ".join(CXXFLAGS + NVCCFLAGS).encode())
    return h.hexdigest()


def _compile(src: Path, obj: Path, deps) -> None:
    stamp = obj.with_suffix(".stamp")
    dig = _digest([src] + list(deps))
    if obj.exists() and stamp.exists() and stamp.read_text() == dig:
        return
    if src.suffix == ".cu":
        cmd = [NVCC] + NVCCFLAGS + ["-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++"] + CXXFLAGS + ["-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    stamp.write_text(dig)


def build(force: bool = False, verbose: bool = False) -> Path:
    OUT_DIR.mkdir(parents=True, exist_ok=True)
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    _embed()
    headers = sorted(CSRC.rglob("*.h")) + sorted(CSRC.rglob("*.hpp")) + sorted(CSRC.rglob("*.cuh"))
    headers.append(PKG.parent / "include" / "linon.h")
    jobs = []
    for rel in CPP_SOURCES + CU_SOURCES:
        src = CSRC / rel
        obj = BUILD_DIR / (rel.replace("/", "_") + ".o")
        jobs.append((src, obj))
    jobs.append((GENERATED, BUILD_DIR / "embedded_sources.o"))
    if force:
        for _, obj in jobs:
            obj.with_suffix(".stamp").unlink(missing_ok=True)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, s, o, headers) for s, o in jobs]
        for f in futs:
            f.result()
    objs = [str(o) for _, o in jobs]
    link_dig = _digest([Path(o) for o in objs])
    stamp = BUILD_DIR / "link.stamp"
    if LIB.exists() and stamp.exists() and stamp.read_text() == link_dig and not force:
        return LIB
    tmp = LIB.with_suffix(".so.tmp")
    cmd = [NVCC, "-shared", "-o", str(tmp)] + objs + ARCH + [
        f"-L{CUDA_HOME / 'lib64'}", "-lnvrtc", "-Xlinker", f"-rpath,{CUDA_HOME / 'lib64'}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    stamp.write_text(link_dig)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
