"""Build liblattice_gpu.so (CUDA, sm_103a) and the drop-in host programs in-tree.

nvcc compiles every translation unit in parallel and links one shared library
next to this file; the host programs link against it with an rpath to this
directory.  FP64 kernels and the detection kernels are compiled with
-fmad=false so that their arithmetic keeps the reference's rounding
(no contraction of a*b+c into one fused operation).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
HOST = PKG / "host"
OBJ = PKG / "_build"
LIB = PKG / "liblattice_gpu.so"
BIN = PKG / "bin"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code never contracts a*b+c into an FMA (gcc does by default on aarch64),
# so host-side arithmetic rounds as the reference's x86 build does.
HOST_FP = ["-Xcompiler", "-ffp-contract=off"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
               "-Xptxas", "-O3"] + HOST_FP

# translation unit -> extra flags
UNITS = {
    "ah_f64.cu": ["-fmad=false"],
    "moore_f64.cu": ["-fmad=false"],
    "detect.cu": ["-fmad=false"],
    "string_length.cu": ["-fmad=false"],
    "snapshot.cu": ["-fmad=false"],
    "boundary.cu": ["-fmad=false"],
    "string_ic.cu": ["-fmad=false"],
    "noalloc.cu": ["-fmad=false"],
    "ah_f64_fast.cu": [],
    "ah_f32.cu": [],
    "moore_f32.cu": [],
    "misc.cu": [],
    "lattice_api.cu": [],
    "batch.cu": [],
    "device_ic.cu": [],
    "tune.cu": [],
    "server.cpp": [],
    "host_ic.cpp": [],
}


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _compile(unit: str, flags: list[str], verbose: bool) -> Path:
    src = CSRC / unit
    out = OBJ / (unit + ".o")
    deps = [src] + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "lattice_gpu.h"]
    if out.exists() and all(out.stat().st_mtime >= d.stat().st_mtime for d in deps) and not os.environ.get("LAT_REBUILD"):
        return out
    cmd = [nvcc()] + ARCH + NVCC_COMMON + flags + ["-c", str(src), "-o", str(out)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-O3", "-std=c++17", "-Xcompiler", "-fPIC"] + HOST_FP + ["-c", str(src), "-o", str(out)]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.run(cmd, check=True)
    return out


def build_library(verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    newest = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest or os.environ.get("LAT_REBUILD"):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    return LIB


def build_programs(verbose: bool = False) -> list[Path]:
    """C++ drop-in programs (host side of the C ABI)."""
    BIN.mkdir(exist_ok=True)
    outs = []
    srcs = sorted(HOST.glob("*_main.cpp"))
    common = [s for s in sorted(HOST.glob("*.cpp")) if not s.name.endswith("_main.cpp")]
    for s in srcs:
        exe = BIN / s.name.replace("_main.cpp", "")
        deps = [s] + common + sorted(HOST.glob("*.hpp")) + [LIB]
        if exe.exists() and all(exe.stat().st_mtime >= d.stat().st_mtime for d in deps):
            outs.append(exe)
            continue
        cmd = ["g++", "-O2", "-std=c++17", "-Wall", "-pthread", "-ffp-contract=off", "-I", str(ROOT / "include"), str(s)] + [str(c) for c in common]
        cmd += ["-L", str(PKG), "-llattice_gpu", "-Wl,-rpath,$ORIGIN/..", "-o", str(exe)]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        outs.append(exe)
    return outs


def build_all(verbose: bool = False) -> None:
    build_library(verbose)
    build_programs(verbose)


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    print(LIB)
