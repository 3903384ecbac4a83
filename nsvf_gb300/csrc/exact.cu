// Compensated re-evaluation of the field at samples that lie far outside
// their voxel.
//
// The reference's inverse-CDF kernel can hand a sample the voxel id of the
// next hit slot after the ray's last one (its tail loop, fairnr/clib/src/
// sample_gpu.cu:188-201, reproduced bit for bit by sample.cu). Such a
// sample's position is many voxels away from that voxel, so its trilinear
// coordinates p = (x - c) / voxel_size + 0.5 reach tens to hundreds and the
// corner weights extrapolate by 1e5 and more. The field's outputs there are
// thousands instead of ~0.01, and any relative rounding error of the field
// (BF16: ~1e-2; FP32: ~1e-6) turns into a colour error of units (BF16) or
// 1e-2 (FP32) on that pixel.
//
// Here those few samples (about 0.01 % of a frame) are evaluated again on
// the CUDA cores in double-float arithmetic: every value is an unevaluated
// sum hi + lo of two FP32 numbers (about 48 significant bits), built from
// the error-free transformations TwoSum (Knuth), FastTwoSum (Dekker) and
// TwoProduct by fused multiply-add, and the dot products of the layers use
// the compensated Dot2 scheme of Ogita, Rump and Oishi ("Accurate sum and
// dot product", SIAM J. Sci. Comput. 26(6), 2005). The sample's position is
// rebuilt from its ray and depth exactly (o + d t as a double-float), then
// interpolation, the five layers and ReLU run in double-float, and the
// (sigma, r, g, b) result is rounded once to FP32 into the field output,
// replacing the tensor-core (or FP32) value before compositing.
//
// The same evaluation decides the pruning mask exactly (nsvf_prune_exact_dev):
// the tensor-core pruning kernel screens every point in BF16 with an error
// scale M (mlp_tc.cu), and only the points it cannot decide -- about 0.3 %
// of a c2 pass -- are evaluated here, their sigma compared with the
// threshold in double-float.
//
// A sample is flagged when any trilinear coordinate leaves [-0.5, 1.5]: half
// a voxel beyond the voxel's faces, well past the x-shift of the reference's
// precomputed centres (voxel_size / 10, fairnr/modules/encoder.py:381-383).
// The tensor-core loaders flag in-kernel (mlp_tc.cu); flag_outliers_kernel
// does it for fields evaluated elsewhere.
#include "common.cuh"

namespace {

constexpr int kThreads = 128;  // one thread per hidden unit
constexpr int kSpb = 4;        // samples per block pass (weight loads shared)
constexpr int E = 32, HID = 128;

struct df {
  float hi, lo;
};

// Knuth's TwoSum: s + e == a + b exactly, for any a, b.
__device__ __forceinline__ df two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}

// Dekker's FastTwoSum, exact when |a| >= |b| (or a == 0).
__device__ __forceinline__ df fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return {s, __fsub_rn(b, __fsub_rn(s, a))};
}

// TwoProduct with a fused multiply-add: p + e == a * b exactly.
__device__ __forceinline__ df two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return {p, __fmaf_rn(a, b, -p)};
}

// Double-float addition with both error terms carried (the accurate
// variant of Hida, Li and Bailey's double-double addition).
__device__ __forceinline__ df df_add(df a, df b) {
  df s = two_sum(a.hi, b.hi);
  const df t = two_sum(a.lo, b.lo);
  s = fast_two_sum(s.hi, __fadd_rn(s.lo, t.hi));
  return fast_two_sum(s.hi, __fadd_rn(s.lo, t.lo));
}

__device__ __forceinline__ df df_neg(df a) { return {-a.hi, -a.lo}; }

__device__ __forceinline__ df df_mul(df a, df b) {
  df p = two_prod(a.hi, b.hi);
  float e = __fmaf_rn(a.hi, b.lo, p.lo);
  e = __fmaf_rn(a.lo, b.hi, e);
  return fast_two_sum(p.hi, e);
}

// a / b for an FP32 divisor: quotient, exact remainder, correction.
__device__ __forceinline__ df df_div_f(df a, float b) {
  const float q1 = __fdiv_rn(a.hi, b);
  const df r = df_add(a, df_neg(two_prod(q1, b)));
  return fast_two_sum(q1, __fdiv_rn(r.hi, b));
}

// Dot2 accumulator: the running sum is p + s, p carrying the leading bits
// and s the accumulated rounding errors of every step.
struct Dot2 {
  float p, s;
  __device__ __forceinline__ void init(float bias) { p = bias; s = 0.0f; }
  // += w * (x.hi + x.lo)
  __device__ __forceinline__ void add(float w, df x) {
    const df h = two_prod(w, x.hi);
    const df q = two_sum(p, h.hi);
    p = q.hi;
    s = __fadd_rn(s, __fadd_rn(q.lo, h.lo));
    s = __fmaf_rn(w, x.lo, s);
  }
  // += a * b with a double-float weight and an FP32 value
  __device__ __forceinline__ void add_df(df a, float v) {
    const df h = two_prod(a.hi, v);
    const df q = two_sum(p, h.hi);
    p = q.hi;
    s = __fadd_rn(s, __fadd_rn(q.lo, h.lo));
    s = __fmaf_rn(a.lo, v, s);
  }
  __device__ __forceinline__ df get() const { return fast_two_sum(p, s); }
};

__device__ __forceinline__ df df_relu(df a) {
  return (a.hi > 0.0f || (a.hi == 0.0f && a.lo > 0.0f)) ? a : df{0.0f, 0.0f};
}

__global__ void __launch_bounds__(256) flag_outliers_kernel(
    int64_t cap, const int64_t *__restrict__ n_dev, const int32_t *__restrict__ vox,
    const float4 *__restrict__ xyzd, int64_t n_vox, float voxel_size,
    const float *__restrict__ centers, int64_t *__restrict__ list,
    unsigned long long *__restrict__ n_list, int64_t list_cap, int32_t *__restrict__ err) {
  int64_t n = cap;
  if (n_dev) n = *n_dev < cap ? *n_dev : cap;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  for (int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; s < n; s += stride) {
    const int64_t v = vox[s];
    if (v < 0 || v >= n_vox) continue;
    const float4 x = xyzd[s];
    // the interpolation's operations (interp.cu)
    const float qx = (x.x - centers[v * 3]) / voxel_size + 0.5f;
    const float qy = (x.y - centers[v * 3 + 1]) / voxel_size + 0.5f;
    const float qz = (x.z - centers[v * 3 + 2]) / voxel_size + 0.5f;
    if (nsvf_far_outside(qx, qy, qz)) nsvf_push_outlier(list, n_list, list_cap, s, err);
  }
}

struct ExactParams {
  int mode;                  // 0: served samples -> out; 1: pruning points -> keep
  // mode 1: row r = v * bits^3 + i is point i of voxel v (offset_points
  // order); keep[v] = 1 if its sigma >= T (rule 1) or > T (rule 0), with T
  // = T_hi + T_lo
  int bits, rule;
  float T_hi, T_lo;
  uint8_t *keep;
  const int64_t *n_rows_dev;
  int64_t rows_cap;
  const int64_t *offset;     // [rows + 1] sample offsets of the rays
  const int64_t *ray_index;  // row -> ray (NULL: identity)
  const float *ray_start;
  int64_t ray_start_stride;  // 3, or 0 for one shared origin
  const float *ray_dir;
  const float *depth;        // [samples] t
  const int32_t *vox;        // [samples]
  int64_t n_vox, n_keys;
  float voxel_size;
  const float *centers;      // [n_vox, 3]
  const int32_t *feats;      // [n_vox, 8]
  const float *values;       // [n_keys, 32]
  const float *wt[5];        // W_l transposed: [K_l, N_l] FP32
  const float *b[5];
  const int64_t *list;
  const unsigned long long *n_list;
  int64_t list_cap;
  float4 *out;               // [samples] (sigma, r, g, b)
  int32_t *err;
  // mode 0, optional: rows whose re-evaluated sample has |r|, |g| or |b|
  // above refine_above are appended to rlist for the FP32 pass
  float refine_above;
  int64_t *rlist;
  unsigned long long *n_rlist;
  int64_t rlist_cap;
};

// Row i of the rays with offset[i] <= s < offset[i + 1] (offsets ascend;
// empty rows share an offset with the next row).
__device__ __forceinline__ int64_t row_of(const int64_t *__restrict__ offset, int64_t rows,
                                          int64_t s) {
  int64_t lo = 0, hi = rows;  // offset[lo] <= s < offset[hi]
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (offset[mid] <= s) lo = mid;
    else hi = mid;
  }
  return lo;
}

// Block pass: kSpb listed samples. Threads 32 j + c (j = sample, c =
// channel) interpolate; then thread n computes hidden unit n of every
// sample, layer by layer, with the activations in shared memory; threads
// 4 j + o compute output o of sample j.
__global__ void __launch_bounds__(kThreads) field_exact_kernel(const ExactParams p) {
  __shared__ float act_hi[kSpb][HID], act_lo[kSpb][HID];
  __shared__ int64_t sample[kSpb], srow[kSpb];
  const int t = threadIdx.x;
  int64_t rows = p.rows_cap;
  if (p.n_rows_dev) rows = *p.n_rows_dev < rows ? *p.n_rows_dev : rows;
  int64_t n = (int64_t)*p.n_list;
  if (n > p.list_cap) n = p.list_cap;
  const int64_t passes = (n + kSpb - 1) / kSpb;
  for (int64_t pass = blockIdx.x; pass < passes; pass += gridDim.x) {
    // interpolation: sample j = t / 32, channel c = t % 32
    {
      const int j = t >> 5, c = t & 31;
      const int64_t li = pass * kSpb + j;
      int64_t s = -1, row = -1;
      df e = {0.0f, 0.0f};
      if (li < n) {
        s = p.list[li];
        int64_t v = -1;
        df x[3];
        if (p.mode == 0) {
          v = s >= 0 ? p.vox[s] : -1;
          if (s >= 0 && v >= 0 && v < p.n_vox && rows > 0) {
            // x = o + d t exactly, as a double-float
            row = row_of(p.offset, rows, s);
            const int64_t ray = p.ray_index ? p.ray_index[row] : row;
            const float tt = p.depth[s];
#pragma unroll
            for (int d = 0; d < 3; ++d) {
              x[d] = two_prod(p.ray_dir[ray * 3 + d], tt);
              x[d] = df_add(x[d], df{p.ray_start[ray * p.ray_start_stride + d], 0.0f});
            }
          } else {
            v = -1;
          }
        } else if (s >= 0) {
          // pruning point: offset_points' FP32 position (the reference's
          // operations: fl(fl(o / (bits - 1)) * hv), then added to the centre)
          const int64_t P = (int64_t)p.bits * p.bits * p.bits;
          v = s / P;
          if (v >= p.n_vox || p.keep[v]) {
            v = -1;   // out of range, or already kept by a certain point
            s = -1;
          } else {
            const int64_t i = s % P;
            const int id[3] = {(int)(i / (p.bits * p.bits)), (int)((i / p.bits) % p.bits),
                               (int)(i % p.bits)};
            const float hv = p.voxel_size / 2.0f, den = (float)(p.bits - 1);
#pragma unroll
            for (int d = 0; d < 3; ++d)
              x[d] = df{__fadd_rn(p.centers[v * 3 + d],
                                  __fmul_rn(__fdiv_rn((float)(2 * id[d] + 1 - p.bits), den), hv)),
                        0.0f};
          }
        }
        if (v >= 0) {
          df q[3];
#pragma unroll
          for (int d = 0; d < 3; ++d) {
            // (x - c) / vs + 0.5
            const df xc = df_add(x[d], df{-p.centers[v * 3 + d], 0.0f});
            q[d] = df_add(df_div_f(xc, p.voxel_size), df{0.5f, 0.0f});
          }
          const df one = {1.0f, 0.0f};
          const df nq[3] = {df_add(one, df_neg(q[0])), df_add(one, df_neg(q[1])),
                            df_add(one, df_neg(q[2]))};
          Dot2 acc;
          acc.init(0.0f);
#pragma unroll
          for (int k = 0; k < 8; ++k) {
            const int64_t key = p.feats[v * 8 + k];
            if (key < 0 || key >= p.n_keys) continue;
            const df w = df_mul(df_mul((k & 4) ? q[0] : nq[0], (k & 2) ? q[1] : nq[1]),
                                (k & 1) ? q[2] : nq[2]);
            acc.add_df(w, __ldg(p.values + key * E + c));
          }
          e = acc.get();
        } else if (s >= 0 && c == 0 && p.err) {
          atomicOr(p.err, 4);
        }
      }
      act_hi[j][c] = e.hi;
      act_lo[j][c] = e.lo;
      if (c == 0) {
        sample[j] = s;
        srow[j] = row;
      }
    }
    __syncthreads();
    // hidden layers 0..3: unit t of every sample
#pragma unroll 1
    for (int l = 0; l < 4; ++l) {
      const int K = l == 0 ? E : HID;
      const float *__restrict__ w = p.wt[l];
      Dot2 acc[kSpb];
      const float bias = p.b[l][t];
#pragma unroll
      for (int j = 0; j < kSpb; ++j) acc[j].init(bias);
#pragma unroll 4
      for (int k = 0; k < K; ++k) {
        const float wk = __ldg(w + (int64_t)k * HID + t);
#pragma unroll
        for (int j = 0; j < kSpb; ++j) acc[j].add(wk, df{act_hi[j][k], act_lo[j][k]});
      }
      __syncthreads();
#pragma unroll
      for (int j = 0; j < kSpb; ++j) {
        const df y = df_relu(acc[j].get());
        act_hi[j][t] = y.hi;
        act_lo[j][t] = y.lo;
      }
      __syncthreads();
    }
    // head: output o of sample j (pruning: sigma only)
    if (t < (p.mode == 0 ? 4 : 1) * kSpb) {
      const int j = p.mode == 0 ? t >> 2 : t, o = p.mode == 0 ? t & 3 : 0;
      const int64_t s = sample[j];
      Dot2 acc;
      acc.init(p.b[4][o]);
      for (int k = 0; k < HID; ++k)
        acc.add(__ldg(p.wt[4] + k * 4 + o), df{act_hi[j][k], act_lo[j][k]});
      const df y = acc.get();
      if (p.mode == 0) {
        // the sample's largest colour magnitude, over its group of 4 lanes
        const float yo = __fadd_rn(y.hi, y.lo);
        float mag = o == 0 ? 0.0f : fabsf(yo);
        mag = fmaxf(mag, __shfl_xor_sync(0x0000ffffu, mag, 1));
        mag = fmaxf(mag, __shfl_xor_sync(0x0000ffffu, mag, 2));
        if (s >= 0) {
          reinterpret_cast<float *>(p.out + s)[o] = yo;
          if (o == 0 && p.n_rlist && srow[j] >= 0 && mag > p.refine_above)
            nsvf_push_outlier(p.rlist, p.n_rlist, p.rlist_cap, srow[j], p.err);
        }
      } else if (s >= 0) {
        {
          // sigma vs T, both normalised double-floats
          const bool above = y.hi > p.T_hi ||
                             (y.hi == p.T_hi && (p.rule == 1 ? y.lo >= p.T_lo : y.lo > p.T_lo));
          if (above) p.keep[s / ((int64_t)p.bits * p.bits * p.bits)] = 1;
        }
      }
    }
    __syncthreads();
  }
}

// FP32 re-evaluation of every sample of the listed rays, except their
// samples far outside the voxel (their double-float values stay). A ray whose
// extrapolated sample has a colour of C puts C times the BF16 error of the
// transmittance in front of it into the pixel; evaluating that ray's other
// samples in FP32 removes that error. Block per listed ray, kRefineSpb samples
// per pass: interpolation (the interpolation kernel's FP32 operations), then
// thread n computes hidden unit n of every sample with the activations in
// shared memory ([k][sample], two float4 broadcasts per k), then 32 threads
// the 4 outputs of the 8 samples.
constexpr int kRefineSpb = 8;

struct RefineParams {
  const int64_t *rlist;
  const unsigned long long *n_rlist;
  int64_t rlist_cap;
  const int64_t *n_rows_dev;
  int64_t rows_cap;
  const int64_t *offset;
  int64_t sample_cap;
  const int32_t *vox;
  const float4 *xyzd;
  int64_t n_vox, n_keys;
  float voxel_size;
  const float *centers;
  const int32_t *feats;
  const float *values;
  const float *wt[5];
  const float *b[5];
  float4 *out;
};

__global__ void __launch_bounds__(kThreads) refine_fp32_kernel(const RefineParams p) {
  __shared__ __align__(16) float act[HID][kRefineSpb];
  __shared__ int64_t sample[kRefineSpb];
  const int t = threadIdx.x;
  int64_t rows = p.rows_cap;
  if (p.n_rows_dev) rows = *p.n_rows_dev < rows ? *p.n_rows_dev : rows;
  int64_t n = (int64_t)*p.n_rlist;
  if (n > p.rlist_cap) n = p.rlist_cap;
  for (int64_t li = blockIdx.x; li < n; li += gridDim.x) {
    const int64_t row = p.rlist[li];
    if (row < 0 || row >= rows) continue;   // uniform over the block
    int64_t a = p.offset[row], e = p.offset[row + 1];
    if (e > p.sample_cap) e = p.sample_cap;
    for (int64_t s0 = a; s0 < e; s0 += kRefineSpb) {
      {
        // sample j = t / 16, channels c and c + 16
        const int j = t >> 4, c = t & 15;
        const int64_t s = s0 + j;
        float e0 = 0.0f, e1 = 0.0f;
        bool use = false;
        if (s < e) {
          const int64_t v = p.vox[s];
          if (v >= 0 && v < p.n_vox) {
            const float4 x = p.xyzd[s];
            const float q[3] = {(x.x - p.centers[v * 3]) / p.voxel_size + 0.5f,
                                (x.y - p.centers[v * 3 + 1]) / p.voxel_size + 0.5f,
                                (x.z - p.centers[v * 3 + 2]) / p.voxel_size + 0.5f};
            use = !nsvf_far_outside(q[0], q[1], q[2]);
#pragma unroll
            for (int k = 0; k < 8; ++k) {
              const int64_t key = p.feats[v * 8 + k];
              if (key < 0 || key >= p.n_keys) continue;
              const float w = ((k & 4) ? q[0] : 1.0f - q[0]) * ((k & 2) ? q[1] : 1.0f - q[1]) *
                              ((k & 1) ? q[2] : 1.0f - q[2]);
              e0 = fmaf(w, __ldg(p.values + key * E + c), e0);
              e1 = fmaf(w, __ldg(p.values + key * E + c + 16), e1);
            }
          }
        }
        act[c][j] = e0;
        act[c + 16][j] = e1;
        if (c == 0) sample[j] = use ? s : -1;
      }
      __syncthreads();
#pragma unroll 1
      for (int l = 0; l < 4; ++l) {
        const int K = l == 0 ? E : HID;
        const float *__restrict__ w = p.wt[l];
        float acc[kRefineSpb];
        const float bias = p.b[l][t];
#pragma unroll
        for (int j = 0; j < kRefineSpb; ++j) acc[j] = bias;
#pragma unroll 4
        for (int k = 0; k < K; ++k) {
          const float wk = __ldg(w + (int64_t)k * HID + t);
          const float4 a0 = reinterpret_cast<const float4 *>(act[k])[0];
          const float4 a1 = reinterpret_cast<const float4 *>(act[k])[1];
          acc[0] = fmaf(wk, a0.x, acc[0]); acc[1] = fmaf(wk, a0.y, acc[1]);
          acc[2] = fmaf(wk, a0.z, acc[2]); acc[3] = fmaf(wk, a0.w, acc[3]);
          acc[4] = fmaf(wk, a1.x, acc[4]); acc[5] = fmaf(wk, a1.y, acc[5]);
          acc[6] = fmaf(wk, a1.z, acc[6]); acc[7] = fmaf(wk, a1.w, acc[7]);
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < kRefineSpb; ++j) act[t][j] = fmaxf(acc[j], 0.0f);
        __syncthreads();
      }
      if (t < 4 * kRefineSpb) {
        const int j = t >> 2, o = t & 3;
        float y = p.b[4][o];
        for (int k = 0; k < HID; ++k) y = fmaf(__ldg(p.wt[4] + k * 4 + o), act[k][j], y);
        const int64_t s = sample[j];
        if (s >= 0) reinterpret_cast<float *>(p.out + s)[o] = y;
      }
      __syncthreads();
    }
  }
}

}  // namespace

extern "C" {

int nsvf_field_refine_fp32_dev(const int64_t *rows, const int64_t *n_rows_list,
                               int64_t rows_list_cap, int64_t rays_cap,
                               const int64_t *n_rays_dev, const int64_t *offset,
                               int64_t sample_cap, const int32_t *voxel, const float *xyz_dist,
                               int64_t n_voxels, int64_t n_keys, float voxel_size,
                               const float *centers, const int32_t *feats, const float *values,
                               const float *const weights_t[5], const float *const biases[5],
                               float *out, void *stream) {
  if (rows_list_cap < 0 || rays_cap < 0 || sample_cap < 0 || n_voxels < 1 || n_keys < 1)
    return NSVF_ERR_INVALID;
  if (rows_list_cap == 0 || rays_cap == 0) return NSVF_OK;
  if (!rows || !n_rows_list || !offset || !voxel || !xyz_dist || !centers || !feats || !values ||
      !weights_t || !biases || !out || (((uintptr_t)xyz_dist) & 15) || (((uintptr_t)out) & 15))
    return NSVF_ERR_INVALID;
  RefineParams p = {};
  for (int l = 0; l < 5; ++l) {
    if (!weights_t[l] || !biases[l]) return NSVF_ERR_INVALID;
    p.wt[l] = weights_t[l];
    p.b[l] = biases[l];
  }
  p.rlist = rows;
  p.n_rlist = (const unsigned long long *)n_rows_list;
  p.rlist_cap = rows_list_cap;
  p.n_rows_dev = n_rays_dev;
  p.rows_cap = rays_cap;
  p.offset = offset;
  p.sample_cap = sample_cap;
  p.vox = voxel;
  p.xyzd = (const float4 *)xyz_dist;
  p.n_vox = n_voxels;
  p.n_keys = n_keys;
  p.voxel_size = voxel_size;
  p.centers = centers;
  p.feats = feats;
  p.values = values;
  p.out = (float4 *)out;
  int64_t blocks = rows_list_cap < 152 * 8 ? rows_list_cap : 152 * 8;
  refine_fp32_kernel<<<(int)blocks, kThreads, 0, (cudaStream_t)stream>>>(p);
  return nsvf_launch_status();
}


int nsvf_flag_outliers(int64_t capacity, const int64_t *n_samples_dev, const int32_t *voxel,
                       const float *xyz_dist, int64_t n_voxels, float voxel_size,
                       const float *centers, int64_t *list, int64_t *n_list, int64_t list_cap,
                       int32_t *err, void *stream) {
  if (capacity < 0 || n_voxels < 1 || list_cap < 0) return NSVF_ERR_INVALID;
  if (capacity == 0) return NSVF_OK;
  if (!voxel || !xyz_dist || !centers || !n_list || (list_cap > 0 && !list) ||
      (((uintptr_t)xyz_dist) & 15))
    return NSVF_ERR_INVALID;
  int blocks = nsvf_grid(capacity, 256);
  if (blocks > 152 * 8) blocks = 152 * 8;
  flag_outliers_kernel<<<blocks, 256, 0, (cudaStream_t)stream>>>(
      capacity, n_samples_dev, voxel, (const float4 *)xyz_dist, n_voxels, voxel_size, centers,
      list, (unsigned long long *)n_list, list_cap, err);
  return nsvf_launch_status();
}

int nsvf_prune_exact_dev(int64_t n_voxels, int bits, int rule, double threshold, int64_t n_keys,
                         float voxel_size, const float *centers, const int32_t *feats,
                         const float *values, const float *const weights_t[5],
                         const float *const biases[5], const int64_t *list,
                         const int64_t *n_list, int64_t list_cap, uint8_t *keep, int32_t *err,
                         void *stream) {
  if (n_voxels < 0 || bits < 2 || bits > 64 || (rule != 0 && rule != 1) || n_keys < 1 ||
      list_cap < 0 || !(threshold > 0.0) || !(threshold < 3.0e38))
    return NSVF_ERR_INVALID;
  if (n_voxels == 0 || list_cap == 0) return NSVF_OK;
  if (!centers || !feats || !values || !weights_t || !biases || !list || !n_list || !keep)
    return NSVF_ERR_INVALID;
  ExactParams p = {};
  for (int l = 0; l < 5; ++l) {
    if (!weights_t[l] || !biases[l]) return NSVF_ERR_INVALID;
    p.wt[l] = weights_t[l];
    p.b[l] = biases[l];
  }
  p.mode = 1;
  p.bits = bits;
  p.rule = rule;
  // T as a normalised double-float
  p.T_hi = (float)threshold;
  p.T_lo = (float)(threshold - (double)p.T_hi);
  p.keep = keep;
  p.n_vox = n_voxels;
  p.n_keys = n_keys;
  p.voxel_size = voxel_size;
  p.centers = centers;
  p.feats = feats;
  p.values = values;
  p.list = list;
  p.n_list = (const unsigned long long *)n_list;
  p.list_cap = list_cap;
  p.rows_cap = 1;
  p.err = err;
  int64_t blocks = (list_cap + kSpb - 1) / kSpb;
  if (blocks > 152 * 8) blocks = 152 * 8;
  field_exact_kernel<<<(int)blocks, kThreads, 0, (cudaStream_t)stream>>>(p);
  return nsvf_launch_status();
}

int nsvf_field_exact_dev(int64_t rows_cap, const int64_t *n_rows_dev, const int64_t *offset,
                         const int64_t *ray_index, const float *ray_start,
                         int64_t ray_start_stride, const float *ray_dir, const float *depth,
                         const int32_t *voxel, int64_t n_voxels, int64_t n_keys,
                         float voxel_size, const float *centers, const int32_t *feats,
                         const float *values, const float *const weights_t[5],
                         const float *const biases[5], const int64_t *list,
                         const int64_t *n_list, int64_t list_cap, float *out,
                         float refine_above, int64_t *refine_rows, int64_t *n_refine_rows,
                         int64_t refine_cap, int32_t *err, void *stream) {
  if (n_refine_rows && (refine_cap < 0 || (refine_cap > 0 && !refine_rows)))
    return NSVF_ERR_INVALID;
  if (rows_cap < 0 || list_cap < 0 || n_voxels < 1 || n_keys < 1 ||
      (ray_start_stride != 0 && ray_start_stride != 3))
    return NSVF_ERR_INVALID;
  if (rows_cap == 0 || list_cap == 0) return NSVF_OK;
  if (!offset || !ray_start || !ray_dir || !depth || !voxel || !centers || !feats || !values ||
      !weights_t || !biases || !list || !n_list || !out || (((uintptr_t)out) & 15))
    return NSVF_ERR_INVALID;
  ExactParams p = {};
  for (int l = 0; l < 5; ++l) {
    if (!weights_t[l] || !biases[l]) return NSVF_ERR_INVALID;
    p.wt[l] = weights_t[l];
    p.b[l] = biases[l];
  }
  p.mode = 0;
  p.n_rows_dev = n_rows_dev;
  p.rows_cap = rows_cap;
  p.offset = offset;
  p.ray_index = ray_index;
  p.ray_start = ray_start;
  p.ray_start_stride = ray_start_stride;
  p.ray_dir = ray_dir;
  p.depth = depth;
  p.vox = voxel;
  p.n_vox = n_voxels;
  p.n_keys = n_keys;
  p.voxel_size = voxel_size;
  p.centers = centers;
  p.feats = feats;
  p.values = values;
  p.list = list;
  p.n_list = (const unsigned long long *)n_list;
  p.list_cap = list_cap;
  p.out = (float4 *)out;
  p.err = err;
  p.refine_above = refine_above;
  p.rlist = refine_rows;
  p.n_rlist = (unsigned long long *)n_refine_rows;
  p.rlist_cap = refine_cap;
  // the listed count is only known on the device: a fixed grid that
  // strides over the passes (idle blocks exit at once)
  int64_t blocks = (list_cap + kSpb - 1) / kSpb;
  if (blocks > 152 * 4) blocks = 152 * 4;
  field_exact_kernel<<<(int)blocks, kThreads, 0, (cudaStream_t)stream>>>(p);
  return nsvf_launch_status();
}

}  // extern "C"
