"""Compile the nsvf_gb300 C-ABI library for sm_103a, in-tree.

``python -m nsvf_gb300.build`` (or ``nsvf_gb300.build.build()``) compiles
every source of nsvf_gb300/csrc/ with nvcc, one process per file in
parallel, into nsvf_gb300/_build/, and links
nsvf_gb300/_build/libnsvf_gb300.so. Only sm_103a code is generated.

Geometry kernels (intersection, sampling) are compiled with -fmad=false
(and their host code with -ffp-contract=off): they spell out every fused
multiply-add the reference's default nvcc build contracts, so their FP32
results are reproducible on a CPU, x86 or Arm.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libnsvf_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          "-I", os.path.join(HERE, "..", "include")]
EXACT_FP = {"intersect.cu", "sample.cu", "chunk.cu", "exact.cu", "svo_grid.cu"}


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _deps():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    files.append(os.path.join(HERE, "..", "include", "nsvf_gb300.h"))
    return max(os.path.getmtime(f) for f in files)


def _compile(src):
    obj = os.path.join(BUILD, src + ".o")
    cmd = [NVCC] + ARCH + COMMON
    if src in EXACT_FP:
        cmd += ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]
    if src.endswith(".cpp"):
        cmd += ["-x", "c++"]
    cmd += ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj


def build(force=False, verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _deps():
        return LIB
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcuda"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
