"""Builds libpartapp_gb300.so (the C-ABI of include/partapp_gb300.h) for sm_103a.

Each CUDA translation unit under csrc/ is compiled by nvcc in parallel, then
linked with the static CUDA runtime into partapp_gb300/_lib/.  The library has
no dependency on torch.  Host code is compiled without floating-point
contraction so the host-side parameter math rounds like the reference;
device code keeps denormals and IEEE division/square root (no fast math).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libpartapp_gb300.so")
HOST = os.path.join(HERE, "host")
CLI = os.path.join(OUT, "partapp_find_obj")
HOST_SOURCES = ["objectdetect_gpu.cpp", "find_obj_main.cpp"]
SOURCES = ["k_stump.cu", "k_unary.cu", "k_msg.cu", "k_reduce.cu", "k_localmax.cu", "k_tc_gemm.cu",
           "k_desc.cu", "k_conv.cu", "pa_api.cu", "pa_noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build partapp_gb300")


def flags() -> list[str]:
    return ARCH + [
        "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
        "-ftz=false", "-prec-div=true", "-prec-sqrt=true",
        "-Xcompiler", "-fPIC,-ffp-contract=off,-fno-fast-math",
        "-I", os.path.join(ROOT, "include"), "-I", CSRC,
    ]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src), os.path.join(ROOT, "include", "partapp_gb300.h")]
    deps += [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    if _stale(obj, deps):
        cmd = [nvcc()] + flags() + extra + ["-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{r.stderr}\n{r.stdout}")
    return obj


def _check_arch() -> None:
    """Objects built on another host architecture are removed, not linked."""
    stamp = os.path.join(OBJ, "ARCH")
    here = platform.machine()
    if os.path.exists(stamp) and open(stamp).read().strip() == here:
        return
    for d in (OBJ, OUT):
        if os.path.isdir(d):
            for f in os.listdir(d):
                os.remove(os.path.join(d, f))
    os.makedirs(OBJ, exist_ok=True)
    with open(stamp, "w") as fh:
        fh.write(here + "\n")


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    """Compile (incrementally) and return the path of the shared library."""
    os.makedirs(OUT, exist_ok=True)
    os.makedirs(OBJ, exist_ok=True)
    _check_arch()
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs + [
            "-lpthread", "-ldl", "-lrt"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr}\n{r.stdout}")
    build_host()
    if verbose:
        print(LIB)
    return LIB


def build_host() -> str:
    """The C++ host layer (partapp_gpu.hpp) and the partapp_find_obj CLI,
    linked against the C-ABI library (rpath $ORIGIN)."""
    srcs = [os.path.join(HOST, s) for s in HOST_SOURCES]
    deps = srcs + [os.path.join(HOST, "partapp_gpu.hpp"), os.path.join(HOST, "mat_io.hpp"), LIB,
                   os.path.join(ROOT, "include", "partapp_gb300.h")]
    if _stale(CLI, deps):
        cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", HOST] + \
            srcs + ["-L", OUT, "-lpartapp_gb300", "-Wl,-rpath,$ORIGIN", "-o", CLI]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host build failed:\n{r.stderr}\n{r.stdout}")
    return CLI


def ptxas_report() -> str:
    """Registers / spills / shared memory of every kernel (-Xptxas -v)."""
    out = []
    for src in SOURCES:
        cmd = [nvcc()] + flags() + ["-Xptxas", "-v", "-c", os.path.join(CSRC, src), "-o",
                                    os.devnull]
        r = subprocess.run(cmd, capture_output=True, text=True)
        out.append(f"== {src}\n{r.stderr}")
    return "\n".join(out)


if __name__ == "__main__":
    if len(sys.argv) > 1 and sys.argv[1] == "--ptxas":
        print(ptxas_report())
    else:
        build(verbose=True)
