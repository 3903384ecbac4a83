// Small kernels that make the served chain free of host synchronisation, so
// that a whole ray chunk can be captured into one CUDA graph:
//   * pinhole ray generation from camera parameters in device memory;
//   * order-preserving compaction of the hit rays (count stays on device);
//   * gather of the hit rays' sorted hit lists with their sampling
//     distribution (probs, steps: fairnr/models/nsvf.py:65-74), and the same
//     distribution for padded rows (the drop-in path).
#include "common.cuh"

namespace {

constexpr int kBlock = 256;

// cam[18] = (origin xyz, camera-to-world rotation R[3][3] row-major with
// columns right/down/forward, focal, cx, cy, width, first pixel, pixel
// count), read on the device so a captured graph can render any chunk of
// any frame. Ray t is pixel first + t (row-major) and looks along
// normalize(R ((j + .5 - cx) / f, (i + .5 - cy) / f, 1)); rays t >= count
// repeat the last pixel with the direction reversed, away from the scene.
// Ray t of a camera's pixel range: local index t (t >= count repeats the last
// pixel, pointing away from the scene), written to slot `out`.
__device__ __forceinline__ void pinhole_ray(const float *__restrict__ cam, int64_t t, int64_t out,
                                            float *__restrict__ ro, float *__restrict__ rd) {
  float f = cam[12], cx = cam[13], cy = cam[14];
  int64_t W = (int64_t)cam[15];
  if (W < 1) W = 1;
  int64_t first = (int64_t)cam[16], count = (int64_t)cam[17];
  if (count < 1) count = 1;
  int64_t pix = first + (t < count ? t : count - 1);
  float j = (float)(pix % W) + 0.5f, i = (float)(pix / W) + 0.5f;
  float a = (j - cx) / f, b = (i - cy) / f;
  float x = cam[3] * a + cam[4] * b + cam[5];
  float y = cam[6] * a + cam[7] * b + cam[8];
  float z = cam[9] * a + cam[10] * b + cam[11];
  float inv = rsqrtf(x * x + y * y + z * z);
  if (t >= count) inv = -inv;
  ro[out * 3 + 0] = cam[0]; ro[out * 3 + 1] = cam[1]; ro[out * 3 + 2] = cam[2];
  rd[out * 3 + 0] = x * inv; rd[out * 3 + 1] = y * inv; rd[out * 3 + 2] = z * inv;
}

__global__ void pinhole_kernel(int64_t n, const float *__restrict__ cam, float *__restrict__ ro,
                               float *__restrict__ rd) {
  int64_t t = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (t >= n) return;
  pinhole_ray(cam, t, t, ro, rd);
}

// A chunk of several pixel ranges (of different frames): segment s (s <
// min(*n_seg, max_seg)) holds cams[s][17] rays, in order; rays past the last
// segment repeat its last pixel pointing away from the scene.
__global__ void pinhole_multi_kernel(int64_t n, int max_seg, const int32_t *__restrict__ n_seg,
                                     const float *__restrict__ cams, float *__restrict__ ro,
                                     float *__restrict__ rd) {
  int64_t t = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (t >= n) return;
  int ns = *n_seg < max_seg ? *n_seg : max_seg;
  if (ns < 1) ns = 1;
  int64_t acc = 0;
  int s = 0;
  for (; s < ns; ++s) {
    int64_t c = (int64_t)cams[s * 18 + 17];
    if (c < 0) c = 0;
    if (t < acc + c) break;
    acc += c;
  }
  if (s == ns) {
    // past the last segment: its last pixel, pointing away
    pinhole_ray(cams + (ns - 1) * 18, (int64_t)1 << 40, t, ro, rd);
    return;
  }
  pinhole_ray(cams + s * 18, t - acc, t, ro, rd);
}

// The hit-row range of every segment of a multi-segment chunk: with scan the
// inclusive prefix sum of the chunk's hit flags, segment s owns hit rows
// [piece_rows[s], piece_rows[s + 1]); segments past *n_seg are empty.
__global__ void piece_rows_kernel(int max_seg, const int32_t *__restrict__ n_seg,
                                  const float *__restrict__ cams, int64_t n,
                                  const int32_t *__restrict__ scan,
                                  int64_t *__restrict__ piece_rows) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const int ns = *n_seg < max_seg ? *n_seg : max_seg;
  int64_t acc = 0;
  piece_rows[0] = 0;
  for (int s = 0; s < max_seg; ++s) {
    if (s < ns) {
      int64_t c = (int64_t)cams[s * 18 + 17];
      acc += c > 0 ? c : 0;
      if (acc > n) acc = n;
    }
    piece_rows[s + 1] = acc > 0 ? (int64_t)scan[acc - 1] : 0;
  }
}

// Rays in the reference's camera convention: ImageReader's eval path
// (fairnr/modules/reader.py:92-119) with get_uv (fairnr/data/data_utils.py:
// 57-65) and get_ray_direction (fairnr/data/geometry.py:116-122).
// cam[20] = fx, fy, cx, cy, inv_RT (3 x 4 camera-to-world, row-major),
// su = W / w, sv = H / h (image read at w x h), w, first pixel. Ray t is
// pixel p = first + t of the w-wide grid (row-major): u = (p % w) su,
// v = (p / w) sv (integer pixel coordinates, no half-pixel offset); the
// point at depth 1 is rt = inv_RT ((u - cx) / fx, (v - cy) / fy, 1, 1), the
// origin is inv_RT's translation and the direction is
// (rt - origin) / (|rt - origin| + 1e-8).
__global__ void camera_rays_kernel(int64_t n, const float *__restrict__ cam,
                                   float *__restrict__ ro, float *__restrict__ rd) {
  int64_t t = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (t >= n) return;
  const float fx = cam[0], fy = cam[1], cx = cam[2], cy = cam[3];
  const float *M = cam + 4;
  const float su = cam[16], sv = cam[17];
  int64_t w = (int64_t)cam[18];
  if (w < 1) w = 1;
  const int64_t p = (int64_t)cam[19] + t;
  const float u = (float)(p % w) * su, v = (float)(p / w) * sv;
  const float x = (u - cx) / fx, y = (v - cy) / fy;
  float d[3];
  for (int k = 0; k < 3; ++k) {
    const float *m = M + 4 * k;
    float pk = m[0] * x + m[1] * y + m[2] + m[3];
    d[k] = pk - m[3];
  }
  const float l = sqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]) + 1e-8f;
  for (int k = 0; k < 3; ++k) {
    ro[t * 3 + k] = M[4 * k + 3];
    rd[t * 3 + k] = d[k] / l;
  }
}

// scan = inclusive prefix sum of hits: hit ray r goes to pix[scan[r] - 1].
__global__ void compact_hits_kernel(int64_t n, const uint8_t *__restrict__ hits,
                                    const int32_t *__restrict__ scan, int64_t *__restrict__ pix,
                                    int64_t *__restrict__ n_hit) {
  int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (r >= n) return;
  if (hits[r]) pix[scan[r] - 1] = r;
  if (r == n - 1) *n_hit = scan[r];
}

// The sampling distribution of one ray (fairnr/models/nsvf.py:65-74): d_k =
// max_k - min_k where slot k is a hit (0 elsewhere), tot = d_0 + d_1 + ... +
// d_{H-1} added one slot at a time in slot order (FP32, the order of a
// plain loop), probs_k = d_k / tot, steps = tot / step. One warp per row:
// the row is read 32 slots at a time (coalesced) and every lane adds the 32
// values in slot order from shuffles, so all lanes hold the same total; a
// second sweep writes the probabilities. Both the drop-in path
// (nsvf_ray_probs) and the served chain (nsvf_gather_probs) use it, so their
// samples are identical.
__device__ __forceinline__ float slot_d(const int32_t *__restrict__ ir,
                                        const float *__restrict__ lr,
                                        const float *__restrict__ hr, int k) {
  return ir[k] == -1 ? 0.0f : __fsub_rn(hr[k], lr[k]);
}

__device__ __forceinline__ float row_total(const int32_t *__restrict__ ir,
                                           const float *__restrict__ lr,
                                           const float *__restrict__ hr, int H, int lane) {
  float tot = 0.0f;
  for (int base = 0; base < H; base += 32) {
    const float dv = base + lane < H ? slot_d(ir, lr, hr, base + lane) : 0.0f;
    const int n = H - base < 32 ? H - base : 32;
    for (int j = 0; j < n; ++j) tot = __fadd_rn(tot, __shfl_sync(0xffffffffu, dv, j));
  }
  return tot;
}

__global__ void __launch_bounds__(kBlock) ray_probs_kernel(
    int64_t rows, int H, float step, const int32_t *__restrict__ idx,
    const float *__restrict__ lo, const float *__restrict__ hi, float *__restrict__ probs,
    float *__restrict__ steps) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (kBlock / 32);
  for (int64_t r = (blockIdx.x * (int64_t)kBlock + threadIdx.x) >> 5; r < rows; r += warps) {
    const int32_t *ir = idx + r * H;
    const float *lr = lo + r * H, *hr = hi + r * H;
    const float tot = row_total(ir, lr, hr, H, lane);
    for (int k = lane; k < H; k += 32) probs[r * H + k] = __fdiv_rn(slot_d(ir, lr, hr, k), tot);
    if (lane == 0) steps[r] = __fdiv_rn(tot, step);
  }
}

// Warp per row i < *n_hit: copy the hit list of ray pix[i] and build its
// sampling distribution with row_total's sum order (the drop-in path's).
// The row is read up to its first -1 only, so it may end there (rows of the
// unpadded leaf-grid sweep): the copy is padded like the sweep pads its rows
// (id -1, depths 10000) and the padded slots' terms (+0) leave the sum
// unchanged, so padded and unpadded rows give the same bits.
__global__ void __launch_bounds__(kBlock) gather_probs_kernel(
    int64_t cap, const int64_t *__restrict__ n_hit, int H, float step,
    const int64_t *__restrict__ pix, const int32_t *__restrict__ idx,
    const float *__restrict__ lo, const float *__restrict__ hi, int32_t *__restrict__ I,
    float *__restrict__ L, float *__restrict__ U, float *__restrict__ probs,
    float *__restrict__ steps) {
  const int lane = threadIdx.x & 31;
  const int64_t n = *n_hit < cap ? *n_hit : cap;
  const int64_t warps = (int64_t)gridDim.x * (kBlock / 32);
  for (int64_t i = (blockIdx.x * (int64_t)kBlock + threadIdx.x) >> 5; i < n; i += warps) {
    const int64_t r = pix[i];
    const int32_t *ir = idx + r * H;
    const float *lr = lo + r * H, *hr = hi + r * H;
    // the valid slots: before the row's first -1
    int cnt = H;
    for (int base = 0; base < H; base += 32) {
      const bool end = base + lane < H && ir[base + lane] == -1;
      const unsigned m = __ballot_sync(0xffffffffu, end);
      if (m) { cnt = base + __ffs(m) - 1; break; }
    }
    float tot = 0.0f;
    for (int base = 0; base < cnt; base += 32) {
      const float dv = base + lane < cnt ? __fsub_rn(hr[base + lane], lr[base + lane]) : 0.0f;
      const int m = cnt - base < 32 ? cnt - base : 32;
      for (int j = 0; j < m; ++j) tot = __fadd_rn(tot, __shfl_sync(0xffffffffu, dv, j));
    }
    for (int k = lane; k < H; k += 32) {
      const bool v = k < cnt;
      const float a = v ? lr[k] : NSVF_MAX_DEPTH_F, b = v ? hr[k] : NSVF_MAX_DEPTH_F;
      I[i * H + k] = v ? ir[k] : -1;
      L[i * H + k] = a;
      U[i * H + k] = b;
      probs[i * H + k] = __fdiv_rn(v ? __fsub_rn(b, a) : 0.0f, tot);
    }
    if (lane == 0) steps[i] = __fdiv_rn(tot, step);
  }
}

}  // namespace

extern "C" {

int nsvf_pinhole_rays(int64_t n, const float *cam, float *ray_start, float *ray_dir,
                      void *stream) {
  if (n < 0 || !cam) return NSVF_ERR_INVALID;
  if (n == 0) return NSVF_OK;
  if (!ray_start || !ray_dir) return NSVF_ERR_INVALID;
  pinhole_kernel<<<nsvf_grid(n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(n, cam, ray_start,
                                                                          ray_dir);
  return nsvf_launch_status();
}

int nsvf_pinhole_rays_multi(int64_t n, int max_seg, const int32_t *n_seg, const float *cams,
                            float *ray_start, float *ray_dir, void *stream) {
  if (n < 0 || max_seg < 1 || !n_seg || !cams) return NSVF_ERR_INVALID;
  if (n == 0) return NSVF_OK;
  if (!ray_start || !ray_dir) return NSVF_ERR_INVALID;
  pinhole_multi_kernel<<<nsvf_grid(n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
      n, max_seg, n_seg, cams, ray_start, ray_dir);
  return nsvf_launch_status();
}

int nsvf_piece_rows(int max_seg, const int32_t *n_seg, const float *cams, int64_t n,
                    const int32_t *scan, int64_t *piece_rows, void *stream) {
  if (max_seg < 1 || n < 1 || !n_seg || !cams || !scan || !piece_rows) return NSVF_ERR_INVALID;
  piece_rows_kernel<<<1, 32, 0, (cudaStream_t)stream>>>(max_seg, n_seg, cams, n, scan, piece_rows);
  return nsvf_launch_status();
}

int nsvf_compact_hits(int64_t n, const uint8_t *hits, const int32_t *scan, int64_t *pix,
                      int64_t *n_hit, void *stream) {
  if (n < 1 || !hits || !scan || !pix || !n_hit) return NSVF_ERR_INVALID;
  compact_hits_kernel<<<nsvf_grid(n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(n, hits, scan, pix,
                                                                               n_hit);
  return nsvf_launch_status();
}

int nsvf_camera_rays(int64_t n, const float *cam, float *ray_start, float *ray_dir,
                     void *stream) {
  if (n < 0 || !cam) return NSVF_ERR_INVALID;
  if (n == 0) return NSVF_OK;
  if (!ray_start || !ray_dir) return NSVF_ERR_INVALID;
  camera_rays_kernel<<<nsvf_grid(n, kBlock), kBlock, 0, (cudaStream_t)stream>>>(n, cam, ray_start,
                                                                               ray_dir);
  return nsvf_launch_status();
}

int nsvf_ray_probs(int64_t rows, int max_hits, float step_size, const int32_t *idx,
                   const float *min_depth, const float *max_depth, float *probs, float *steps,
                   void *stream) {
  if (rows < 0 || max_hits < 1) return NSVF_ERR_INVALID;
  if (rows == 0) return NSVF_OK;
  if (!idx || !min_depth || !max_depth || !probs || !steps) return NSVF_ERR_INVALID;
  int blocks = nsvf_grid(rows, kBlock / 32);
  if (blocks > 152 * 16) blocks = 152 * 16;
  ray_probs_kernel<<<blocks, kBlock, 0, (cudaStream_t)stream>>>(rows, max_hits, step_size, idx,
                                                               min_depth, max_depth, probs, steps);
  return nsvf_launch_status();
}

int nsvf_gather_probs(int64_t cap, const int64_t *n_hit, int max_hits, float step_size,
                      const int64_t *pix, const int32_t *idx, const float *min_depth,
                      const float *max_depth, int32_t *out_idx, float *out_min, float *out_max,
                      float *probs, float *steps, void *stream) {
  if (cap < 0 || max_hits < 1 || !n_hit) return NSVF_ERR_INVALID;
  if (cap == 0) return NSVF_OK;
  if (!pix || !idx || !min_depth || !max_depth || !out_idx || !out_min || !out_max || !probs ||
      !steps)
    return NSVF_ERR_INVALID;
  // warp per row, grid-stride over at most 16 blocks per SM (the row count is
  // only known on the device)
  int blocks = nsvf_grid(cap, kBlock / 32);
  if (blocks > 152 * 16) blocks = 152 * 16;
  gather_probs_kernel<<<blocks, kBlock, 0, (cudaStream_t)stream>>>(
      cap, n_hit, max_hits, step_size, pix, idx, min_depth, max_depth, out_idx, out_min, out_max,
      probs, steps);
  return nsvf_launch_status();
}

}  // extern "C"
