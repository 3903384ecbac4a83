// Front-to-back transmittance compositing and its backward.
//
// Reference: VolumeRenderer.forward_chunk (fairnr/modules/renderer.py:193-218):
//   a_i = 1 - exp(-fe_i)                      (probability the sample is not empty)
//   T_i = exp(-sum_{j<i} fe_j)                (shifted cumulative sum in FP32)
//   p_i = a_i * T_i, depth = sum p_i t_i, missed = 1 - sum p_i,
//   color = sum p_i * tex_i.
// One warp composites one ray: lanes take 32 consecutive samples at a time,
// a shuffle scan builds the prefix of fe, and the running sum is carried
// from one 32-sample chunk to the next. `kahan` switches the carried prefix
// to a compensated (Kahan) sum.
//
// Backward, with g_i = dL/dp_i + dL/ddepth * t_i + <dL/dcolor, tex_i> - dL/dmissed:
//   dL/dfe_j  = g_j * exp(-fe_j) * T_j - sum_{i>j} g_i p_i
//   dL/dtex_i = dL/dcolor * p_i
#include <cstdint>

#include "common.cuh"

namespace {

constexpr int kWarps = 8;

struct Prefix {
  float s, c;  // running sum and Kahan compensation
};

__device__ __forceinline__ float warp_incl_scan(float x, int lane) {
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    float y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

__device__ __forceinline__ float warp_sum(float x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Exclusive prefix of fe for this lane's sample given the carried prefix of
// the previous chunks; advances the carry by the chunk total.
__device__ __forceinline__ float chunk_prefix(float fe, int lane, Prefix &carry, bool kahan) {
  float incl = warp_incl_scan(fe, lane);
  float excl = incl - fe;
  float total = __shfl_sync(0xffffffffu, incl, 31);
  float pre;
  if (kahan) {
    pre = carry.s + (excl - carry.c);
    float y = total - carry.c;
    float t = carry.s + y;
    carry.c = (t - carry.s) - y;
    carry.s = t;
  } else {
    pre = carry.s + excl;
    carry.s += total;
  }
  return pre;
}

__global__ void __launch_bounds__(kWarps * 32) composite_fwd_kernel(
    int64_t rays, int M, const float *__restrict__ fe, const float *__restrict__ tex,
    const float *__restrict__ t, float *__restrict__ probs, float *__restrict__ depth,
    float *__restrict__ missed, float *__restrict__ color, int kahan) {
  int lane = threadIdx.x & 31;
  int64_t r = blockIdx.x * (int64_t)kWarps + (threadIdx.x >> 5);
  if (r >= rays) return;
  const float *F = fe + r * M;
  Prefix carry{0.f, 0.f};
  float sp = 0.f, sd = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f;
  for (int base = 0; base < M; base += 32) {
    int i = base + lane;
    bool in = i < M;
    float f = in ? F[i] : 0.f;
    float pre = chunk_prefix(f, lane, carry, kahan != 0);
    float p = in ? (1.0f - expf(-f)) * expf(-pre) : 0.f;
    if (in) {
      if (probs) probs[r * M + i] = p;
      sp += p;
      if (t) sd += p * t[r * M + i];
      if (tex) {
        const float *x = tex + (r * M + i) * 3;
        c0 += p * x[0]; c1 += p * x[1]; c2 += p * x[2];
      }
    }
  }
  sp = warp_sum(sp);
  sd = warp_sum(sd);
  c0 = warp_sum(c0); c1 = warp_sum(c1); c2 = warp_sum(c2);
  if (lane == 0) {
    if (depth) depth[r] = sd;
    if (missed) missed[r] = 1.0f - sp;
    if (color) { color[r * 3 + 0] = c0; color[r * 3 + 1] = c1; color[r * 3 + 2] = c2; }
  }
}

__global__ void __launch_bounds__(kWarps * 32) composite_bwd_kernel(
    int64_t rays, int M, const float *__restrict__ fe, const float *__restrict__ tex,
    const float *__restrict__ t, const float *__restrict__ g_probs,
    const float *__restrict__ g_depth, const float *__restrict__ g_missed,
    const float *__restrict__ g_color, float *__restrict__ g_fe, float *__restrict__ g_tex,
    int kahan) {
  int lane = threadIdx.x & 31;
  int64_t r = blockIdx.x * (int64_t)kWarps + (threadIdx.x >> 5);
  if (r >= rays) return;
  const float *F = fe + r * M;
  float gd = g_depth ? g_depth[r] : 0.f;
  float gm = g_missed ? g_missed[r] : 0.f;
  float gc0 = 0.f, gc1 = 0.f, gc2 = 0.f;
  if (g_color) { gc0 = g_color[r * 3]; gc1 = g_color[r * 3 + 1]; gc2 = g_color[r * 3 + 2]; }
  // pass 1: total = sum_i g_i p_i
  Prefix carry{0.f, 0.f};
  float total = 0.f;
  for (int base = 0; base < M; base += 32) {
    int i = base + lane;
    bool in = i < M;
    float f = in ? F[i] : 0.f;
    float pre = chunk_prefix(f, lane, carry, kahan != 0);
    if (in) {
      float p = (1.0f - expf(-f)) * expf(-pre);
      float g = (g_probs ? g_probs[r * M + i] : 0.f) - gm;
      if (t) g += gd * t[r * M + i];
      if (tex) {
        const float *x = tex + (r * M + i) * 3;
        g += gc0 * x[0] + gc1 * x[1] + gc2 * x[2];
      }
      total += g * p;
    }
  }
  total = warp_sum(total);
  // pass 2: suffix_j = total - inclusive prefix of g p
  carry = Prefix{0.f, 0.f};
  float gp_carry = 0.f;
  for (int base = 0; base < M; base += 32) {
    int i = base + lane;
    bool in = i < M;
    float f = in ? F[i] : 0.f;
    float pre = chunk_prefix(f, lane, carry, kahan != 0);
    float T = expf(-pre);
    float e = expf(-f);
    float p = in ? (1.0f - e) * T : 0.f;
    float g = 0.f;
    if (in) {
      g = (g_probs ? g_probs[r * M + i] : 0.f) - gm;
      if (t) g += gd * t[r * M + i];
      if (tex) {
        const float *x = tex + (r * M + i) * 3;
        g += gc0 * x[0] + gc1 * x[1] + gc2 * x[2];
      }
    }
    float gp = g * p;
    float incl = warp_incl_scan(gp, lane) + gp_carry;
    gp_carry = __shfl_sync(0xffffffffu, incl, 31);
    if (in) {
      g_fe[r * M + i] = g * e * T - (total - incl);
      if (g_tex) {
        float *y = g_tex + (r * M + i) * 3;
        y[0] = gc0 * p; y[1] = gc1 * p; y[2] = gc2 * p;
      }
    }
  }
}

// Served path: compositing of compacted samples. Ray r owns samples
// [offset[r], offset[r+1]) (its valid samples in depth order); field[s] =
// (sigma, r, g, b), xyzd[s].w = distance, depth[s]. Writes pixel pix[r] of
// the frame: color = sum p c + missed * bg, depth = sum p t + missed *
// bg_depth, missed. fe = relu(sigma) * dist * sigma_scale as the reference
// renderer (fairnr/modules/renderer.py:117-121).
__global__ void __launch_bounds__(kWarps * 32) composite_segments_kernel(
    int64_t rays, const int64_t *__restrict__ offset, const float4 *__restrict__ field,
    const float4 *__restrict__ xyzd, const float *__restrict__ depth,
    const int64_t *__restrict__ pix, float sigma_scale, float bg_r, float bg_g, float bg_b,
    float bg_depth, float *__restrict__ out_color, float *__restrict__ out_depth,
    float *__restrict__ out_missed, int kahan, const int64_t *__restrict__ n_dev,
    int64_t sample_cap) {
  int lane = threadIdx.x & 31;
  int64_t r = blockIdx.x * (int64_t)kWarps + (threadIdx.x >> 5);
  if (n_dev) {
    int64_t nd = *n_dev;
    if (nd < rays) rays = nd < 0 ? 0 : nd;
  }
  if (r >= rays) return;
  // the ray's segment, clamped to the sample buffers (a frame whose samples
  // overflowed them is composited again; nothing is read past them)
  const int64_t e = offset[r + 1] < sample_cap ? offset[r + 1] : sample_cap;
  const int64_t a = offset[r] < e ? offset[r] : e, n = e - a;
  Prefix carry{0.f, 0.f};
  float sp = 0.f, sd = 0.f, c0 = 0.f, c1 = 0.f, c2 = 0.f;
  for (int64_t base = 0; base < n; base += 32) {
    int64_t i = base + lane;
    bool in = i < n;
    float4 f = in ? field[a + i] : make_float4(0.f, 0.f, 0.f, 0.f);
    float dist = in ? xyzd[a + i].w : 0.f;
    float fe = (fmaxf(f.x, 0.0f) * dist) * sigma_scale;
    float pre = chunk_prefix(fe, lane, carry, kahan != 0);
    if (in) {
      float p = (1.0f - expf(-fe)) * expf(-pre);
      sp += p;
      sd += p * depth[a + i];
      c0 += p * f.y; c1 += p * f.z; c2 += p * f.w;
    }
  }
  sp = warp_sum(sp);
  sd = warp_sum(sd);
  c0 = warp_sum(c0); c1 = warp_sum(c1); c2 = warp_sum(c2);
  if (lane == 0) {
    int64_t q = pix[r];
    float missed = 1.0f - sp;
    out_color[q * 3 + 0] = c0 + missed * bg_r;
    out_color[q * 3 + 1] = c1 + missed * bg_g;
    out_color[q * 3 + 2] = c2 + missed * bg_b;
    out_depth[q] = sd + missed * bg_depth;
    out_missed[q] = missed;
  }
}

}  // namespace

extern "C" {

int nsvf_composite_segments(int64_t rays, const int64_t *offset, const float *field,
                            const float *xyz_dist, const float *depth, const int64_t *pixel,
                            float sigma_scale, const float bg[3], float bg_depth,
                            float *out_color, float *out_depth, float *out_missed, int kahan,
                            void *stream) {
  if (rays < 0 || !bg) return NSVF_ERR_INVALID;
  if (rays == 0) return NSVF_OK;
  if (!offset || !field || !xyz_dist || !depth || !pixel || !out_color || !out_depth ||
      !out_missed || ((((uintptr_t)field) | ((uintptr_t)xyz_dist)) & 15))
    return NSVF_ERR_INVALID;
  composite_segments_kernel<<<nsvf_grid(rays, kWarps), kWarps * 32, 0, (cudaStream_t)stream>>>(
      rays, offset, (const float4 *)field, (const float4 *)xyz_dist, depth, pixel, sigma_scale,
      bg[0], bg[1], bg[2], bg_depth, out_color, out_depth, out_missed, kahan, nullptr, INT64_MAX);
  return nsvf_launch_status();
}

int nsvf_composite_segments_dev(int64_t rays_cap, const int64_t *n_rays_dev,
                                const int64_t *offset, int64_t sample_cap, const float *field,
                                const float *xyz_dist, const float *depth, const int64_t *pixel,
                                float sigma_scale, const float bg[3], float bg_depth,
                                float *out_color, float *out_depth, float *out_missed, int kahan,
                                void *stream) {
  if (rays_cap < 0 || sample_cap < 0 || !bg || !n_rays_dev) return NSVF_ERR_INVALID;
  if (rays_cap == 0) return NSVF_OK;
  if (!offset || !field || !xyz_dist || !depth || !pixel || !out_color || !out_depth ||
      !out_missed || ((((uintptr_t)field) | ((uintptr_t)xyz_dist)) & 15))
    return NSVF_ERR_INVALID;
  composite_segments_kernel<<<nsvf_grid(rays_cap, kWarps), kWarps * 32, 0, (cudaStream_t)stream>>>(
      rays_cap, offset, (const float4 *)field, (const float4 *)xyz_dist, depth, pixel, sigma_scale,
      bg[0], bg[1], bg[2], bg_depth, out_color, out_depth, out_missed, kahan, n_rays_dev,
      sample_cap);
  return nsvf_launch_status();
}


int nsvf_composite(int64_t rays, int max_steps, const float *free_energy, const float *texture,
                   const float *sampled_depth, float *probs, float *depth, float *missed,
                   float *colors, int kahan, void *stream) {
  if (rays < 0 || max_steps < 0 || (rays > 0 && max_steps > 0 && !free_energy))
    return NSVF_ERR_INVALID;
  if (rays == 0) return NSVF_OK;
  composite_fwd_kernel<<<nsvf_grid(rays, kWarps), kWarps * 32, 0, (cudaStream_t)stream>>>(
      rays, max_steps, free_energy, texture, sampled_depth, probs, depth, missed, colors, kahan);
  return nsvf_launch_status();
}

int nsvf_composite_backward(int64_t rays, int max_steps, const float *free_energy,
                            const float *texture, const float *sampled_depth,
                            const float *grad_probs, const float *grad_depth,
                            const float *grad_missed, const float *grad_colors,
                            float *grad_free_energy, float *grad_texture, int kahan,
                            void *stream) {
  if (rays < 0 || max_steps < 0 || (rays > 0 && max_steps > 0 && (!free_energy || !grad_free_energy)))
    return NSVF_ERR_INVALID;
  if ((grad_depth && !sampled_depth) || (grad_colors && !texture)) return NSVF_ERR_INVALID;
  if (rays == 0) return NSVF_OK;
  composite_bwd_kernel<<<nsvf_grid(rays, kWarps), kWarps * 32, 0, (cudaStream_t)stream>>>(
      rays, max_steps, free_energy, texture, sampled_depth, grad_probs, grad_depth, grad_missed,
      grad_colors, grad_free_energy, grad_texture, kahan);
  return nsvf_launch_status();
}

}  // extern "C"
