"""Build the reference's own ray/voxel code for the CPU, into oracle/_ref/.

TEST INFRASTRUCTURE ONLY. This recipe runs only where the reference checkout
exists (it reads /root/reference in place and never copies its sources into
the repository); everything it writes goes to oracle/_ref/, which git ignores.
Its outputs pin the C oracle (oracle/clib_oracle.c) and generate the golden
fixtures under tests/golden/.

Two artefacts:

* ``oracle/_ref/libref_clib.so``: the reference's CUDA kernel bodies from
  fairnr/clib/src/intersect_gpu.cu and fairnr/clib/src/sample_gpu.cu compiled
  as plain C++. The kernel part of each file (everything before the first
  ``*_kernel_wrapper`` host function, whose ``<<<>>>`` launch a C++ compiler
  cannot parse) is cut into oracle/_ref/*.inc at build time and compiled
  against oracle/ref_shim/cuda_utils.h, which stands in for the CUDA
  built-ins. ``-mfma -ffp-contract=fast`` makes g++ contract ``a + b * c`` into
  a fused multiply-add where nvcc's default ``-fmad=true`` does.
* ``oracle/_ref/octree/ref_octree*.so``: fairnr/clib/src/octree.cpp (the
  reference's own CPU octree builder) compiled as a CPU torch extension with
  a 5-line binding (oracle/ref_shim/octree_binding.cpp). The reference file
  omits ``<queue>`` and ``<cassert>``; they are force-included.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# Where this recipe reads the reference checkout: NSVF_REFERENCE_ROOT, else
# the checkout's location in the container that builds the fixtures (the
# only place in the repository that names it; oracle.ref_import uses REF).
REF = os.environ.get("NSVF_REFERENCE_ROOT") or "/root/reference"
OUT = os.path.join(HERE, "_ref")
CLIB = os.path.join(REF, "fairnr", "clib")


def available():
    return os.path.isdir(CLIB)


def _cut_kernels(src, dst):
    """Copy the lines of `src` that precede its first kernel-wrapper function."""
    with open(src) as f:
        lines = f.readlines()
    keep = []
    for line in lines:
        if line.startswith("void ") and "_kernel_wrapper(" in line:
            break
        keep.append(line)
    with open(dst, "w") as f:
        f.writelines(keep)


def build_clib():
    os.makedirs(OUT, exist_ok=True)
    so = os.path.join(OUT, "libref_clib.so")
    inter = os.path.join(OUT, "intersect_kernels.inc")
    samp = os.path.join(OUT, "sample_kernels.inc")
    _cut_kernels(os.path.join(CLIB, "src", "intersect_gpu.cu"), inter)
    _cut_kernels(os.path.join(CLIB, "src", "sample_gpu.cu"), samp)
    cmd = [
        "g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-mfma", "-ffp-contract=fast", "-w",
        "-I", os.path.join(HERE, "ref_shim"),
        "-I", os.path.join(CLIB, "include"),
        "-I", "/usr/local/cuda/include",
        '-DREF_INTERSECT_KERNELS="%s"' % inter,
        '-DREF_SAMPLE_KERNELS="%s"' % samp,
        os.path.join(HERE, "ref_shim", "ref_entry.cc"),
        "-o", so,
    ]
    subprocess.check_call(cmd)
    return so


def build_octree():
    from torch.utils.cpp_extension import load
    bdir = os.path.join(OUT, "octree")
    os.makedirs(bdir, exist_ok=True)
    return load(
        name="ref_octree",
        sources=[os.path.join(CLIB, "src", "octree.cpp"),
                 os.path.join(HERE, "ref_shim", "octree_binding.cpp")],
        extra_include_paths=[os.path.join(CLIB, "include"), "/usr/local/cuda/include"],
        extra_cflags=["-O2", "-w", "-include", "queue", "-include", "cassert"],
        build_directory=bdir,
        verbose=False,
    )


def build():
    if not available():
        print("oracle/build_ref.py: reference checkout not found; nothing built", file=sys.stderr)
        return False
    build_clib()
    build_octree()
    return True


if __name__ == "__main__":
    build()
