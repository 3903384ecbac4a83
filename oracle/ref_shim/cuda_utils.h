/*
 * Host-only stand-in for the reference's fairnr/clib/include/cuda_utils.h,
 * used ONLY by oracle/build_ref.py to compile the reference's CUDA kernel
 * bodies as plain C++ on the CPU (test infrastructure, never shipped).
 *
 * It provides what the kernel bodies use from a CUDA device: the
 * blockIdx/threadIdx/blockDim built-ins (set by the caller before it calls a
 * kernel function as an ordinary C++ function), __fdividef (IEEE division
 * here; the GPU intrinsic is an approximate reciprocal), and empty function
 * qualifiers.
 */
#pragma once
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <queue>
#include <cuda_runtime.h>

#undef __global__
#undef __device__
#undef __host__
#define __global__
#define __device__
#define __host__

struct ref_cpu_idx { unsigned int x, y, z; };
extern ref_cpu_idx threadIdx, blockIdx, blockDim;

static inline float __fdividef(float a, float b) { return a / b; }
using std::max;
using std::min;
