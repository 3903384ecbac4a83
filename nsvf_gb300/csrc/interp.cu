// Trilinear interpolation of voxel-corner embeddings and its backward
// (embedding scatter with vectorised atomics).
//
// Reference: SparseVoxelEncoder.forward (fairnr/modules/encoder.py:578-590)
// with trilinear_interp (fairnr/data/geometry.py:195-200): for a sample x in
// voxel v with centre c, p = (x - c) / voxel_size + 0.5, corner k = 4*ix +
// 2*iy + iz (offset_points order) has weight prod_d (q_kd ? p_d : 1 - p_d)
// and emb = sum_k w_k * values[feats[v, k]]. The reference materialises the
// 8 gathered rows per sample ([Ns, 8, E]) with two F.embedding calls; here
// one thread produces 4 channels of one sample from 8 float4 loads, and the
// 8 threads of a sample read each 128-byte corner row together.
#include "common.cuh"

namespace {

constexpr int kBlock = 256;

// w_k for corner k from p (q_kd in {0,1}: p*q + (1-p)*(1-q) reduces to p or
// 1-p exactly), multiplied in dimension order like torch's prod.
__device__ __forceinline__ float corner_w(const float p[3], int k) {
  float a = (k & 4) ? p[0] : 1.0f - p[0];
  float b = (k & 2) ? p[1] : 1.0f - p[1];
  float c = (k & 1) ? p[2] : 1.0f - p[2];
  return a * b * c;
}

// Voxel ids outside [0, n_vox) and corner ids outside [0, n_keys) are not
// read: the sample's embedding is 0 there and bit 2 of *err is set.
template <typename IdxT, typename FeatT>
__global__ void __launch_bounds__(kBlock) trilinear_fwd_kernel(
    int64_t ns, int e4, float voxel_size, int64_t n_vox, int64_t n_keys,
    const IdxT *__restrict__ sidx, const float *__restrict__ xyz, const float *__restrict__ centers,
    const FeatT *__restrict__ feats, const float4 *__restrict__ values, float4 *__restrict__ emb,
    int32_t *__restrict__ err) {
  int64_t t = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  int64_t s = t / e4;
  int ch = (int)(t - s * e4);
  if (s >= ns) return;
  int64_t v = (int64_t)sidx[s];
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  if (v < 0 || v >= n_vox) {
    emb[s * e4 + ch] = acc;
    if (err && ch == 0) atomicOr(err, 4);
    return;
  }
  float p[3];
#pragma unroll
  for (int d = 0; d < 3; ++d) p[d] = (xyz[s * 3 + d] - centers[v * 3 + d]) / voxel_size + 0.5f;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    int64_t key = (int64_t)feats[v * 8 + k];
    if (key < 0 || key >= n_keys) {
      if (err) atomicOr(err, 4);
      continue;
    }
    float w = corner_w(p, k);
    float4 x = __ldg(values + key * e4 + ch);
    acc.x = fmaf(w, x.x, acc.x); acc.y = fmaf(w, x.y, acc.y);
    acc.z = fmaf(w, x.z, acc.z); acc.w = fmaf(w, x.w, acc.w);
  }
  emb[s * e4 + ch] = acc;
}

// Backward: grad_values[feats[v, k]] += w_k * g (float4 atomics), and
// optionally grad_xyz = sum_k dw_k/dx . <values_k, g>.
template <typename IdxT, typename FeatT>
__global__ void __launch_bounds__(kBlock) trilinear_bwd_kernel(
    int64_t ns, int e4, float voxel_size, int64_t n_vox, int64_t n_keys,
    const IdxT *__restrict__ sidx, const float *__restrict__ xyz, const float *__restrict__ centers,
    const FeatT *__restrict__ feats, const float4 *__restrict__ values,
    const float4 *__restrict__ grad_emb, float4 *__restrict__ grad_values,
    float *__restrict__ grad_xyz) {
  int64_t t = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  int64_t s = t / e4;
  int ch = (int)(t - s * e4);
  bool live = s < ns;
  float gx = 0.f, gy = 0.f, gz = 0.f;
  int64_t v = live ? (int64_t)sidx[s] : -1;
  if (v < 0 || v >= n_vox) live = false;
  if (live) {
    float p[3];
#pragma unroll
    for (int d = 0; d < 3; ++d) p[d] = (xyz[s * 3 + d] - centers[v * 3 + d]) / voxel_size + 0.5f;
    float4 g = grad_emb[s * e4 + ch];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      int64_t key = (int64_t)feats[v * 8 + k];
      if (key < 0 || key >= n_keys) continue;
      float w = corner_w(p, k);
      if (grad_values) atomicAdd(grad_values + key * e4 + ch, make_float4(w * g.x, w * g.y, w * g.z, w * g.w));
      if (grad_xyz) {
        float4 x = __ldg(values + key * e4 + ch);
        float dot = x.x * g.x + x.y * g.y + x.z * g.z + x.w * g.w;
        float a = (k & 4) ? p[0] : 1.0f - p[0];
        float b = (k & 2) ? p[1] : 1.0f - p[1];
        float c = (k & 1) ? p[2] : 1.0f - p[2];
        float sa = (k & 4) ? 1.0f : -1.0f, sb = (k & 2) ? 1.0f : -1.0f, sc = (k & 1) ? 1.0f : -1.0f;
        gx += dot * sa * b * c;
        gy += dot * a * sb * c;
        gz += dot * a * b * sc;
      }
    }
  }
  if (grad_xyz) {
    // the e4 threads of a sample are consecutive lanes: reduce over them
    unsigned mask = 0xffffffffu;
    for (int o = 1; o < e4 && o < 32; o <<= 1) {
      gx += __shfl_xor_sync(mask, gx, o);
      gy += __shfl_xor_sync(mask, gy, o);
      gz += __shfl_xor_sync(mask, gz, o);
    }
    if (s < ns && ch == 0) {
      float inv = 1.0f / voxel_size;
      grad_xyz[s * 3 + 0] = gx * inv;
      grad_xyz[s * 3 + 1] = gy * inv;
      grad_xyz[s * 3 + 2] = gz * inv;
    }
  }
}

struct InterpArgs {
  int64_t ns;
  int e;
  float vs;
  int64_t n_vox, n_keys;
  const void *sidx;
  const float *xyz, *centers;
  const void *feats;
  const float *values;
};

template <typename IdxT, typename FeatT>
int launch_fwd(const InterpArgs &a, float *emb, int32_t *err, cudaStream_t s) {
  int e4 = a.e / 4;
  trilinear_fwd_kernel<IdxT, FeatT><<<nsvf_grid(a.ns * e4, kBlock), kBlock, 0, s>>>(
      a.ns, e4, a.vs, a.n_vox, a.n_keys, (const IdxT *)a.sidx, a.xyz, a.centers,
      (const FeatT *)a.feats, (const float4 *)a.values, (float4 *)emb, err);
  return nsvf_launch_status();
}

template <typename IdxT, typename FeatT>
int launch_bwd(const InterpArgs &a, const float *grad_emb, float *grad_values, float *grad_xyz,
               cudaStream_t s) {
  int e4 = a.e / 4;
  trilinear_bwd_kernel<IdxT, FeatT><<<nsvf_grid(a.ns * e4, kBlock), kBlock, 0, s>>>(
      a.ns, e4, a.vs, a.n_vox, a.n_keys, (const IdxT *)a.sidx, a.xyz, a.centers,
      (const FeatT *)a.feats, (const float4 *)a.values, (const float4 *)grad_emb,
      (float4 *)grad_values, grad_xyz);
  return nsvf_launch_status();
}

// embed_dim / 4 must be a power of two <= 32 (E in {4, 8, ..., 128}) so the
// threads of one sample are aligned lanes of one warp.
bool bad_args(int64_t ns, int e, int idx_bytes, int feat_bytes) {
  int e4 = e / 4;
  return ns < 0 || e < 4 || (e % 4) != 0 || (e4 & (e4 - 1)) != 0 || e4 > 32 ||
         (idx_bytes != 4 && idx_bytes != 8) || (feat_bytes != 4 && feat_bytes != 8);
}

}  // namespace

extern "C" {

int nsvf_trilinear_embed(int64_t n_samples, int embed_dim, float voxel_size, int64_t n_voxels,
                         int64_t n_keys, const void *sampled_idx, int idx_bytes, const float *xyz,
                         const float *centers, const void *feats, int feat_bytes,
                         const float *values, float *emb, int32_t *err, void *stream) {
  if (bad_args(n_samples, embed_dim, idx_bytes, feat_bytes)) return NSVF_ERR_INVALID;
  if (n_samples == 0) return NSVF_OK;
  if (!sampled_idx || !xyz || !centers || !feats || !values || !emb) return NSVF_ERR_INVALID;
  if ((((uintptr_t)values) | ((uintptr_t)emb)) & 15) return NSVF_ERR_INVALID;
  InterpArgs a{n_samples, embed_dim, voxel_size, n_voxels, n_keys, sampled_idx, xyz, centers,
               feats, values};
  cudaStream_t s = (cudaStream_t)stream;
  if (idx_bytes == 8 && feat_bytes == 8) return launch_fwd<int64_t, int64_t>(a, emb, err, s);
  if (idx_bytes == 8) return launch_fwd<int64_t, int32_t>(a, emb, err, s);
  if (feat_bytes == 8) return launch_fwd<int32_t, int64_t>(a, emb, err, s);
  return launch_fwd<int32_t, int32_t>(a, emb, err, s);
}

int nsvf_trilinear_embed_backward(int64_t n_samples, int embed_dim, float voxel_size,
                                  int64_t n_voxels, int64_t n_keys, const void *sampled_idx,
                                  int idx_bytes, const float *xyz, const float *centers,
                                  const void *feats, int feat_bytes, const float *values,
                                  const float *grad_emb, float *grad_values, float *grad_xyz,
                                  void *stream) {
  if (bad_args(n_samples, embed_dim, idx_bytes, feat_bytes)) return NSVF_ERR_INVALID;
  if (n_samples == 0) return NSVF_OK;
  if (!sampled_idx || !xyz || !centers || !feats || !grad_emb || (!grad_values && !grad_xyz) ||
      (grad_xyz && !values))
    return NSVF_ERR_INVALID;
  if ((((uintptr_t)grad_emb) | ((uintptr_t)grad_values) | ((uintptr_t)values)) & 15)
    return NSVF_ERR_INVALID;
  InterpArgs a{n_samples, embed_dim, voxel_size, n_voxels, n_keys, sampled_idx, xyz, centers,
               feats, values};
  cudaStream_t s = (cudaStream_t)stream;
  if (idx_bytes == 8 && feat_bytes == 8)
    return launch_bwd<int64_t, int64_t>(a, grad_emb, grad_values, grad_xyz, s);
  if (idx_bytes == 8) return launch_bwd<int64_t, int32_t>(a, grad_emb, grad_values, grad_xyz, s);
  if (feat_bytes == 8) return launch_bwd<int32_t, int64_t>(a, grad_emb, grad_values, grad_xyz, s);
  return launch_bwd<int32_t, int32_t>(a, grad_emb, grad_values, grad_xyz, s);
}

}  // extern "C"
