"""Builds the CUDA library libmhd_gb300.so in-tree for sm_103a.

The translation units below are compiled in parallel with nvcc and linked
into one shared library next to this file:
  csrc/mhd_fp64.cu  plain FP64 kernels, --fmad=false (bit-exact arithmetic)
  csrc/mhd_fp32.cu  FP32 reconstruction/flux kernels (contraction allowed, FP32
                    denormals flushed, approximate FP32 division and square root)
  csrc/mhd_capi.cu  the extern "C" boundary of include/mhd_gb300.h
  csrc/mhd_surrogate.cu  surrogate data, training and evaluation kernels
                    (--fmad=false: its FP64 labels match the CPU IMC bit for bit)
  csrc/mhd_noalloc.cu  the allocation-free time step
  csrc/mhd_peak.cu  the FP64 throughput measurement (the plain path's roofline)
  csrc/mhd_gravity.cu  self-gravity: FFT + tridiagonal potential solve, the half kicks
  csrc/mhd_io.cpp   host code: the reference's output and restart files
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmhd_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
          "--expt-relaxed-constexpr", "-I", os.path.join(HERE, "..", "include")]
UNITS = {
    "mhd_fp64.cu": ["--fmad=false"],
    "mhd_fp32.cu": ["--fmad=true", "-ftz=true", "-prec-div=false", "-prec-sqrt=false"],
    "mhd_capi.cu": ["--fmad=false"],
    "mhd_surrogate.cu": ["--fmad=false"],
    "mhd_noalloc.cu": ["--fmad=false"],
    "mhd_peak.cu": [],
    "mhd_gravity.cu": [],
    "mhd_io.cpp": [],
}


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmhd_gb300.so")
    return exe


def _sources():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cuh", ".h", ".cpp"))]
    inc = os.path.join(HERE, "..", "include")
    deps += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return deps


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(s) <= t for s in _sources())


def build(force=False, verbose=False, extra=()):
    """Compile and link; returns the library path."""
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    exe = nvcc()
    procs = []
    objs = []
    for src, flags in UNITS.items():
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = [exe, *ARCH, *COMMON, *flags, *extra, "-c", path, "-o", obj]
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        procs.append((cmd, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
        objs.append(obj)
    failed = []
    for cmd, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((cmd, out.decode(errors="replace")))
        elif verbose and out:
            print(out.decode(errors="replace"), file=sys.stderr)
    if failed:
        msg = "\n".join(" ".join(c) + "\n" + o for c, o in failed)
        raise RuntimeError("nvcc failed:\n" + msg)
    tmp = LIB + ".tmp"
    cmd = [exe, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
    print(LIB)
