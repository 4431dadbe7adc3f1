"""Build libsphgb300.so in-tree with nvcc for sm_103a.

Three translation units compile in parallel:
  sph_f64.cu  FP64 engine, --fmad=false (every product/sum rounded separately,
              as the reference computes, so FP64 results match bit for bit)
  sph_f32.cu  FP32 engine, multiply-add contraction on
  sph_capi.cu C ABI, runtime, checkpoint schedule
Host code is compiled with -ffp-contract=off for the same reason. Nothing is
architecture specific on the host side (the GPU machine is aarch64).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libsphgb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC,-ffp-contract=off,-fvisibility=hidden"]
SOURCES = {
    "sph_f64.cu": ["--fmad=false"],
    "sph_f32.cu": ["--fmad=true"],
    "sph_capi.cu": [],
    "sph_noalloc.cu": ["--fmad=false"],
    "sph_server.cu": [],
    "sph_design.cu": ["--fmad=false"],
}
DEPS = ["sph_common.cuh", "sph_fixed.cuh", "sph_kernels.cuh", "sph_coop.cuh", "sph_engine.cuh", "sph_pack.cuh",
        "sph_iface.hpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build sphadjoint_gb300")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    files = [os.path.join(CSRC, f) for f in list(SOURCES) + DEPS]
    files.append(os.path.join(HERE, "..", "include", "sphadjoint_gb300.h"))
    files.append(os.path.abspath(__file__))
    return any(os.path.getmtime(f) > t for f in files if os.path.exists(f))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    procs = []
    objs = []
    for src, extra in SOURCES.items():
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        procs.append((src, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for src, p in procs:
        out, _ = p.communicate()
        if verbose or p.returncode:
            sys.stderr.write(out.decode(errors="replace"))
        if p.returncode:
            failed.append(src)
    if failed:
        raise RuntimeError("nvcc failed for " + ", ".join(failed))
    tmp = LIB + ".tmp"
    subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
