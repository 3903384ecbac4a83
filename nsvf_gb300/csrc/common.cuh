// Shared device helpers for the nsvf_gb300 kernels (sm_103a).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/nsvf_gb300.h"

#define NSVF_MAX_DEPTH_F 10000.0f

// Process-wide count of kernels launched by this library (nsvf_launch_count).
void nsvf_count_launch();

// Launch-status helper, called right after each kernel launch: counts it and
// turns the launch error into a status (never exits).
static inline int nsvf_launch_status() {
  nsvf_count_launch();
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? NSVF_OK : NSVF_ERR_CUDA;
}

static inline int nsvf_grid(int64_t work, int block) {
  int64_t g = (work + block - 1) / block;
  if (g < 1) g = 1;
  if (g > 0x7fffffff) g = 0x7fffffff;
  return (int)g;
}

// Slab test of a ray (origin o, reciprocal direction inv) against the cube of
// centre c and half size h. Same operations, in the same order, as the
// reference's RayAABBIntersection (fairnr/clib/src/intersect_gpu.cu:73-122):
// per axis two subtractions and one product per bound, a swap, then the
// running max/min with t starting in [0, 1e5]. The reference exits early when
// an axis already separates; the running interval only shrinks, so testing
// lo > hi once at the end gives the same verdict and the same (lo, hi).
// Comparisons with NaN are false, so a NaN axis leaves the interval unchanged.
__device__ __forceinline__ bool nsvf_slab(float ox, float oy, float oz, float ix, float iy,
                                          float iz, float cx, float cy, float cz, float h,
                                          float &t_lo, float &t_hi) {
  float lo = 0.0f, hi = 100000.0f;
  float l, u;
  l = __fmul_rn(__fsub_rn(__fsub_rn(cx, h), ox), ix);
  u = __fmul_rn(__fsub_rn(__fadd_rn(cx, h), ox), ix);
  if (u < l) { float t = l; l = u; u = t; }
  lo = (l > lo) ? l : lo;
  hi = (u < hi) ? u : hi;
  l = __fmul_rn(__fsub_rn(__fsub_rn(cy, h), oy), iy);
  u = __fmul_rn(__fsub_rn(__fadd_rn(cy, h), oy), iy);
  if (u < l) { float t = l; l = u; u = t; }
  lo = (l > lo) ? l : lo;
  hi = (u < hi) ? u : hi;
  l = __fmul_rn(__fsub_rn(__fsub_rn(cz, h), oz), iz);
  u = __fmul_rn(__fsub_rn(__fadd_rn(cz, h), oz), iz);
  if (u < l) { float t = l; l = u; u = t; }
  lo = (l > lo) ? l : lo;
  hi = (u < hi) ? u : hi;
  t_lo = lo;
  t_hi = hi;
  return !(lo > hi);
}

// nsvf_slab for a ray whose direction has no zero component (every
// reciprocal finite and nonzero), with the same result bit for bit and about
// half the compare/select work. s = +1 where the reciprocal is >= 0, else -1.
//  * No NaN can occur, and for each axis rounding is monotone, so
//    fl(fl(c - h) - o) * inv <= fl(fl(c + h) - o) * inv when inv > 0 (and >=
//    when inv < 0): the reference's swap is decided by the sign alone. near =
//    fl(c - s h) and far = fl(c + s h) are the reference's bounds, swapped
//    when inv < 0 (s h is exact).
//  * lo only grows from +0 and is never -0; max(lo, l + 0) equals
//    (l > lo ? l : lo) for every non-NaN l (l + 0 turns -0 into +0).
//  * hi keeps the compare/select: a -0 that becomes hi must stay -0.
__device__ __forceinline__ bool nsvf_slab_fast(float ox, float oy, float oz, float ix, float iy,
                                               float iz, float sx, float sy, float sz, float cx,
                                               float cy, float cz, float h, float &t_lo,
                                               float &t_hi) {
  float lo = 0.0f, hi = 100000.0f;
  float l, u, sh;
  sh = __fmul_rn(sx, h);
  l = __fmul_rn(__fsub_rn(__fsub_rn(cx, sh), ox), ix);
  u = __fmul_rn(__fsub_rn(__fadd_rn(cx, sh), ox), ix);
  lo = fmaxf(lo, __fadd_rn(l, 0.0f));
  hi = (u < hi) ? u : hi;
  sh = __fmul_rn(sy, h);
  l = __fmul_rn(__fsub_rn(__fsub_rn(cy, sh), oy), iy);
  u = __fmul_rn(__fsub_rn(__fadd_rn(cy, sh), oy), iy);
  lo = fmaxf(lo, __fadd_rn(l, 0.0f));
  hi = (u < hi) ? u : hi;
  sh = __fmul_rn(sz, h);
  l = __fmul_rn(__fsub_rn(__fsub_rn(cz, sh), oz), iz);
  u = __fmul_rn(__fsub_rn(__fadd_rn(cz, sh), oz), iz);
  lo = fmaxf(lo, __fadd_rn(l, 0.0f));
  hi = (u < hi) ? u : hi;
  t_lo = lo;
  t_hi = hi;
  return !(lo > hi);
}

// A sample lies far outside its voxel when a trilinear coordinate p = (x -
// c) / voxel_size + 0.5 leaves [-0.5, 1.5] (half a voxel past a face). Its
// corner weights then extrapolate, and the field there is re-evaluated in
// compensated arithmetic (exact.cu). NaN coordinates are not flagged.
__device__ __forceinline__ bool nsvf_far_outside(float qx, float qy, float qz) {
  return fabsf(__fsub_rn(qx, 0.5f)) > 1.0f || fabsf(__fsub_rn(qy, 0.5f)) > 1.0f ||
         fabsf(__fsub_rn(qz, 0.5f)) > 1.0f;
}

// Appends sample s to a device list (count *n_list, capacity list_cap); a
// full list sets bit 4 (16) of *err.
__device__ __forceinline__ void nsvf_push_outlier(int64_t *list, unsigned long long *n_list,
                                                  int64_t list_cap, int64_t s, int32_t *err) {
  const unsigned long long k = atomicAdd(n_list, 1ull);
  if ((int64_t)k < list_cap) list[k] = s;
  else if (err) atomicOr(err, 16);
}

// Correctly rounded reciprocal (the reference uses the approximate
// __fdividef(1, d); see the note in include/nsvf_gb300.h).
__device__ __forceinline__ float nsvf_rcp(float d) { return __frcp_rn(d); }
