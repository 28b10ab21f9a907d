"""Builds the in-tree CUDA library ``cable_gb300/lib/libcablegpu.so`` for
sm_103a (GB300) with nvcc.  No CPU fallback exists: without this library the
package refuses to run."""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIBDIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIBDIR, "libcablegpu.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

SOURCES = ["cablegpu.cu", "phase_a.cu", "phase_b.cu", "phase_c1.cu", "phase_c2.cu", "phase_c3.cu", "tables.cpp",
           "surrogate.cu", "cgio.cpp"]
# Per-file extra flags: the canopy phase is FP32-only and division-heavy, so
# it uses the approximate division / exp intrinsics, without implicit
# multiply-add contraction (-fmad=false: its instantiations -- diagnostics,
# surrogate, harvest, coupled -- must compute bit-identical results, and the
# compiler's contraction choices depend on the surrounding code; its hot
# arithmetic has explicit multiply-adds instead); radiation, soil heat and
# soil water use the approximate (2 ulp) FP32 division, keeping IEEE square
# root and denormals (their state updates are error-free double-FP32 or
# FP64, and the correction-form solves are insensitive to ulp-level
# coefficient errors); the snow pack keeps IEEE division, since its layering
# thresholds turn ulp differences into branch flips more often than the
# reference's own FP32 build does.  CG_MAXNREG caps registers per thread
# (CG_MAXNREG_S64: of the soil kernels' FP64-solve instantiations),
# chosen per kernel from measured step times at 4M tiles (radiation 80, soil
# heat 80, canopy 72, soil water 112, snow pack 128; FP64 solves: soil heat
# 80, soil water 96, where the FP64 recursion's latency wants the warps),
# trading a few hundred bytes of spills for occupancy; the
# block size itself is a launch-time choice (autotuned).
EXTRA_FLAGS = {
    "phase_a.cu": ["-prec-div=false", "-DCG_MAXNREG=80"],
    "phase_b.cu": ["--use_fast_math", "-fmad=false", "-DCG_MAXNREG=72"],
    "phase_c1.cu": ["-DCG_MAXNREG=128"],
    "phase_c2.cu": ["-prec-div=false", "-DCG_MAXNREG=80", "-DCG_MAXNREG_S64=80"],
    "phase_c3.cu": ["-prec-div=false", "-DCG_MAXNREG=112", "-DCG_MAXNREG_S64=96"],
}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build cable_gb300")


def sources():
    return [os.path.join(CSRC, s) for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def _deps():
    deps = sources() + [os.path.abspath(__file__)]   # compiler flags live here
    for d in (CSRC, INCLUDE):
        deps += [os.path.join(d, f) for f in os.listdir(d) if f.endswith((".h", ".cuh", ".hpp"))]
    return deps


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile (if needed) and return the library path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()
    objs, procs = [], []
    flags = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I" + INCLUDE] + ARCH
    for src in sources():
        obj = os.path.join(LIBDIR, os.path.basename(src) + ".o")
        objs.append(obj)
        cmd = [nvcc] + flags + EXTRA_FLAGS.get(os.path.basename(src), []) + ["-c", src, "-o", obj]
        if verbose:
            print(" ".join(cmd))
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            raise RuntimeError("nvcc failed: %s\n%s" % (" ".join(cmd), out.decode(errors="replace")))
    tmp = LIB + ".tmp"
    subprocess.run([nvcc, "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart"], check=True)
    os.replace(tmp, LIB)
    for o in objs:
        os.remove(o)
    return LIB


if __name__ == "__main__":
    print(build(force=True, verbose=True))
