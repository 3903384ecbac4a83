// Ray-voxel intersection kernels: brute-force AABB, sparse-voxel octree
// (plain and with the encoder's depth sort fused), and ray-ball.
//
// Reference behaviour: fairnr/clib/src/intersect_gpu.cu:15-237 (kernels) and
// fairnr/clib/src/intersect.cpp:15-112 (allocation: idx -1, depths 0).
// Design: one thread per ray over the flattened [b*m] ray list (the reference
// launches one block of <= 512 threads per batch row and copies the voxel set
// or octree into every row: fairnr/clib/__init__.py:62-71, 101-111). Here
// every ray batch reads ONE copy of the voxels/octree, which stays resident in
// L2 (c2 scene: 277,580 nodes x 48 B = 13 MB of a 129 MB L2).
#include <atomic>

#include "common.cuh"

namespace {

constexpr int kRayBlock = 128;

// ---------------------------------------------------------------- AABB ----

// Voxel centres are staged through shared memory in tiles; a block stops
// scanning once every ray in it has n_max hits.
constexpr int kAabbTile = 1024;

__global__ void __launch_bounds__(kRayBlock) aabb_kernel(
    int b, int b_pts, int n, int m, float hv, int n_max, const float *__restrict__ ray_start,
    const float *__restrict__ ray_dir, const float *__restrict__ points, int32_t *__restrict__ idx,
    float *__restrict__ min_depth, float *__restrict__ max_depth) {
  __shared__ float sc[kAabbTile * 3];
  // A block covers rays of one batch row only, so the voxel set is uniform.
  int blocks_per_row = (m + kRayBlock - 1) / kRayBlock;
  int g = blockIdx.x / blocks_per_row;
  int j = (blockIdx.x % blocks_per_row) * kRayBlock + threadIdx.x;
  bool live = j < m;
  int64_t r = (int64_t)g * m + j;
  const float *P = points + (b_pts == 1 ? 0 : (int64_t)g * n * 3);
  float ox = 0, oy = 0, oz = 0, ix = 0, iy = 0, iz = 0;
  if (live) {
    ox = ray_start[r * 3 + 0]; oy = ray_start[r * 3 + 1]; oz = ray_start[r * 3 + 2];
    ix = nsvf_rcp(ray_dir[r * 3 + 0]); iy = nsvf_rcp(ray_dir[r * 3 + 1]);
    iz = nsvf_rcp(ray_dir[r * 3 + 2]);
  }
  int cnt = 0;
  int32_t *I = idx + r * n_max;
  float *LO = min_depth + r * n_max, *HI = max_depth + r * n_max;
  for (int base = 0; base < n; base += kAabbTile) {
    int tile = min(kAabbTile, n - base);
    if (__syncthreads_and(!live || cnt >= n_max)) break;
    for (int t = threadIdx.x; t < tile * 3; t += kRayBlock) sc[t] = P[(int64_t)base * 3 + t];
    __syncthreads();
    if (live) {
      for (int k = 0; k < tile && cnt < n_max; ++k) {
        float lo, hi;
        if (nsvf_slab(ox, oy, oz, ix, iy, iz, sc[k * 3], sc[k * 3 + 1], sc[k * 3 + 2], hv, lo, hi)) {
          I[cnt] = base + k; LO[cnt] = lo; HI[cnt] = hi; ++cnt;
        }
      }
    }
    __syncthreads();
  }
  if (live) {
    for (int l = cnt; l < n_max; ++l) { I[l] = -1; LO[l] = 0.0f; HI[l] = 0.0f; }
  }
}

// ----------------------------------------------------------------- SVO ----

// Packed octree node: box = (cx, cy, cz, +-half) with a negative half marking
// a leaf (children[8] == 1), kids = the 8 child ids.
struct PackedTree {
  float4 *box;   // [b_pts * n]
  int4 *kids;    // [b_pts * n * 2]
};

__global__ void pack_octree_kernel(int64_t total, float hv, const float *__restrict__ points,
                                   const int32_t *__restrict__ children, float4 *__restrict__ box,
                                   int4 *__restrict__ kids) {
  int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (k >= total) return;
  const int32_t *c = children + k * 9;
  int size = c[8];
  float h = __fmul_rn(hv, (float)size);
  box[k] = make_float4(points[k * 3 + 0], points[k * 3 + 1], points[k * 3 + 2],
                       size == 1 ? -h : h);
  kids[k * 2 + 0] = make_int4(c[0], c[1], c[2], c[3]);
  kids[k * 2 + 1] = make_int4(c[4], c[5], c[6], c[7]);
}

constexpr int kSvoStack = 256;

// Depth-first traversal with the reference's visiting order. The reference
// pushes every existing child untested and tests a node when it pops it; here
// the children of a hit node are tested when the node is expanded and only
// the hit ones are pushed (children 0..7, so child 7 is popped first). The
// set of tests and the order of emitted leaves are the same; the stack holds
// at most 1 + 7 * levels entries instead of 1 + 7 * levels + untested ones.
template <bool SORTED>
__global__ void __launch_bounds__(kRayBlock) svo_kernel(
    int64_t rays, int m, int b_pts, int n, int n_max, const float *__restrict__ ray_start,
    const float *__restrict__ ray_dir, const float4 *__restrict__ box_all,
    const int4 *__restrict__ kids_all, int32_t *__restrict__ idx, float *__restrict__ min_depth,
    float *__restrict__ max_depth, uint8_t *__restrict__ hits, int32_t *__restrict__ err) {
  int64_t r = blockIdx.x * (int64_t)kRayBlock + threadIdx.x;
  if (r >= rays) return;
  int64_t g = (b_pts == 1) ? 0 : r / m;
  const float4 *box = box_all + g * n;
  const int4 *kids = kids_all + g * n * 2;
  float ox = ray_start[r * 3 + 0], oy = ray_start[r * 3 + 1], oz = ray_start[r * 3 + 2];
  float ix = nsvf_rcp(ray_dir[r * 3 + 0]), iy = nsvf_rcp(ray_dir[r * 3 + 1]),
        iz = nsvf_rcp(ray_dir[r * 3 + 2]);
  int32_t *I = idx + r * n_max;
  float *LO = min_depth + r * n_max, *HI = max_depth + r * n_max;

  // SORTED keeps the hits in (thread-local) arrays and insertion-sorts them.
  constexpr int kMaxSorted = SORTED ? 128 : 1;
  int32_t hid[kMaxSorted];
  float hlo[kMaxSorted], hhi[kMaxSorted];

  int cnt = 0;
  int stack[kSvoStack];
  int sp = 0;
  {
    float4 rb = box[n - 1];
    float lo, hi;
    if (nsvf_slab(ox, oy, oz, ix, iy, iz, rb.x, rb.y, rb.z, fabsf(rb.w), lo, hi))
      stack[sp++] = n - 1;
  }
  // A well-formed octree pops every node at most once per ray; more pops, a
  // child id outside [0, n) or a full stack mean a malformed input, which is
  // reported through `err` instead of looping or reading out of bounds.
  int64_t pops = 0;
  bool bad = false;
  while (sp > 0 && cnt < n_max) {
    if (++pops > n) { bad = true; break; }
    int k = stack[--sp];
    float4 kb = box[k];
    if (kb.w < 0.0f) {  // leaf: recompute its interval (same inputs, same bits)
      float lo, hi;
      nsvf_slab(ox, oy, oz, ix, iy, iz, kb.x, kb.y, kb.z, -kb.w, lo, hi);
      if (SORTED) {
        int p = cnt;
        while (p > 0 && hlo[p - 1] > lo) {
          hid[p] = hid[p - 1]; hlo[p] = hlo[p - 1]; hhi[p] = hhi[p - 1]; --p;
        }
        hid[p] = k; hlo[p] = lo; hhi[p] = hi;
      } else {
        I[cnt] = k; LO[cnt] = lo; HI[cnt] = hi;
      }
      ++cnt;
      continue;
    }
    int4 ka = kids[k * 2 + 0], kc = kids[k * 2 + 1];
    int ch[8] = {ka.x, ka.y, ka.z, ka.w, kc.x, kc.y, kc.z, kc.w};
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      int c = ch[u];
      if (c > -1) {
        if (c >= n) { bad = true; continue; }
        float4 cb = box[c];
        float lo, hi;
        if (nsvf_slab(ox, oy, oz, ix, iy, iz, cb.x, cb.y, cb.z, fabsf(cb.w), lo, hi)) {
          if (sp < kSvoStack) stack[sp++] = c;
          else bad = true;
        }
      }
    }
  }
  if (bad && err) atomicOr(err, 1);
  if (SORTED) {
    // Emulate "misses -> 10000, sort all n_max slots by min_depth" with ties
    // resolved by slot: hits with lo <= 10000 first, then the misses, then
    // any hit beyond 10000.
    int split = 0;
    while (split < cnt && !(hlo[split] > NSVF_MAX_DEPTH_F)) ++split;
    int o = 0;
    for (int p = 0; p < split; ++p, ++o) { I[o] = hid[p]; LO[o] = hlo[p]; HI[o] = hhi[p]; }
    for (int p = cnt; p < n_max; ++p, ++o) { I[o] = -1; LO[o] = NSVF_MAX_DEPTH_F; HI[o] = NSVF_MAX_DEPTH_F; }
    for (int p = split; p < cnt; ++p, ++o) { I[o] = hid[p]; LO[o] = hlo[p]; HI[o] = hhi[p]; }
    hits[r] = cnt > 0;
  } else {
    for (int l = cnt; l < n_max; ++l) { I[l] = -1; LO[l] = 0.0f; HI[l] = 0.0f; }
  }
}

// ---------------------------------------------------------------- ball ----

__global__ void __launch_bounds__(kRayBlock) ball_kernel(
    int64_t rays, int m, int b_pts, int n, float radius, int n_max,
    const float *__restrict__ ray_start, const float *__restrict__ ray_dir,
    const float *__restrict__ points, int32_t *__restrict__ idx, float *__restrict__ min_depth,
    float *__restrict__ max_depth) {
  int64_t r = blockIdx.x * (int64_t)kRayBlock + threadIdx.x;
  if (r >= rays) return;
  const float *P = points + ((b_pts == 1) ? 0 : (r / m) * (int64_t)n * 3);
  float x0 = ray_start[r * 3 + 0], y0 = ray_start[r * 3 + 1], z0 = ray_start[r * 3 + 2];
  float xw = ray_dir[r * 3 + 0], yw = ray_dir[r * 3 + 1], zw = ray_dir[r * 3 + 2];
  float r2max = __fmul_rn(radius, radius);
  int32_t *I = idx + r * n_max;
  float *LO = min_depth + r * n_max, *HI = max_depth + r * n_max;
  int cnt = 0;
  for (int k = 0; k < n && cnt < n_max; ++k) {
    float x = __fsub_rn(P[k * 3 + 0], x0), y = __fsub_rn(P[k * 3 + 1], y0),
          z = __fsub_rn(P[k * 3 + 2], z0);
    float d2 = __fmaf_rn(z, z, __fmaf_rn(y, y, __fmul_rn(x, x)));
    float proj = __fmaf_rn(z, zw, __fmaf_rn(y, yw, __fmul_rn(x, xw)));
    float p2 = __fmul_rn(proj, proj);
    float r2 = __fsub_rn(d2, p2);
    if (r2 < r2max) {
      float depth = __fsqrt_rn(p2);
      float blur = __fsqrt_rn(__fsub_rn(r2max, r2));
      I[cnt] = k; LO[cnt] = __fsub_rn(depth, blur); HI[cnt] = __fadd_rn(depth, blur); ++cnt;
    }
  }
  for (int l = cnt; l < n_max; ++l) { I[l] = -1; LO[l] = 0.0f; HI[l] = 0.0f; }
}

// Ray pointers may be NULL when there are no rays (empty tensors).
bool bad_common(int b, int b_pts, int n, int m, int n_max, const void *a, const void *c,
                const void *d) {
  bool no_rays = (int64_t)b * m == 0;
  return b < 0 || m < 0 || n < 1 || n_max < 1 || (b_pts != 1 && b_pts != b) ||
         (!no_rays && (!a || !c)) || !d;
}

}  // namespace

static std::atomic<long long> g_launches{0};
void nsvf_count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }

extern "C" {

long long nsvf_launch_count(void) { return g_launches.load(std::memory_order_relaxed); }

const char *nsvf_status_string(int status) {
  switch (status) {
    case NSVF_OK: return "ok";
    case NSVF_ERR_INVALID: return "invalid argument";
    case NSVF_ERR_CUDA: return "CUDA error";
    case NSVF_ERR_OCTREE: return "malformed octree";
    case NSVF_ERR_CAPACITY: return "output capacity too small";
    default: return "unknown status";
  }
}

int nsvf_aabb_intersect(int b, int b_pts, int n, int m, float voxelsize, int n_max,
                        const float *ray_start, const float *ray_dir, const float *points,
                        int32_t *idx, float *min_depth, float *max_depth, void *stream) {
  if (bad_common(b, b_pts, n, m, n_max, ray_start, ray_dir, points)) return NSVF_ERR_INVALID;
  if ((int64_t)b * m == 0) return NSVF_OK;
  if (!idx || !min_depth || !max_depth) return NSVF_ERR_INVALID;
  int blocks_per_row = (m + kRayBlock - 1) / kRayBlock;
  int64_t grid = (int64_t)b * blocks_per_row;
  if (grid > 0x7fffffff) return NSVF_ERR_INVALID;
  aabb_kernel<<<(int)grid, kRayBlock, 0, (cudaStream_t)stream>>>(
      b, b_pts, n, m, voxelsize * 0.5f, n_max, ray_start, ray_dir, points, idx,
      min_depth, max_depth);
  return nsvf_launch_status();
}

int64_t nsvf_svo_workspace_bytes(int b_pts, int n) {
  return (int64_t)b_pts * n * (int64_t)(sizeof(float4) + 2 * sizeof(int4));
}

static int svo_launch(bool sorted, int b, int b_pts, int n, int m, float voxelsize, int n_max,
                      const float *ray_start, const float *ray_dir, const float *points,
                      const int32_t *children, int32_t *idx, float *min_depth, float *max_depth,
                      uint8_t *hits, int32_t *err, void *workspace, void *stream) {
  if (bad_common(b, b_pts, n, m, n_max, ray_start, ray_dir, points) || !children || !workspace ||
      (sorted && n_max > 128))
    return NSVF_ERR_INVALID;
  if ((int64_t)b * m > 0 && (!idx || !min_depth || !max_depth || (sorted && !hits)))
    return NSVF_ERR_INVALID;
  if (((uintptr_t)workspace) & 15) return NSVF_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  int64_t total = (int64_t)b_pts * n;
  float4 *box = (float4 *)workspace;
  int4 *kids = (int4 *)(box + total);
  float hv = voxelsize * 0.5f;
  pack_octree_kernel<<<nsvf_grid(total, 256), 256, 0, s>>>(total, hv, points, children, box, kids);
  nsvf_count_launch();
  int64_t rays = (int64_t)b * m;
  if (rays == 0) return nsvf_launch_status();
  if (sorted)
    svo_kernel<true><<<nsvf_grid(rays, kRayBlock), kRayBlock, 0, s>>>(
        rays, m, b_pts, n, n_max, ray_start, ray_dir, box, kids, idx, min_depth, max_depth, hits,
        err);
  else
    svo_kernel<false><<<nsvf_grid(rays, kRayBlock), kRayBlock, 0, s>>>(
        rays, m, b_pts, n, n_max, ray_start, ray_dir, box, kids, idx, min_depth, max_depth, hits,
        err);
  return nsvf_launch_status();
}

int nsvf_svo_intersect(int b, int b_pts, int n, int m, float voxelsize, int n_max,
                       const float *ray_start, const float *ray_dir, const float *points,
                       const int32_t *children, int32_t *idx, float *min_depth,
                       float *max_depth, int32_t *err, void *workspace, void *stream) {
  return svo_launch(false, b, b_pts, n, m, voxelsize, n_max, ray_start, ray_dir, points, children,
                    idx, min_depth, max_depth, nullptr, err, workspace, stream);
}

int nsvf_svo_intersect_sorted(int b, int b_pts, int n, int m, float voxelsize, int n_max,
                              const float *ray_start, const float *ray_dir, const float *points,
                              const int32_t *children, int32_t *idx, float *min_depth,
                              float *max_depth, uint8_t *hits, int32_t *err, void *workspace,
                              void *stream) {
  return svo_launch(true, b, b_pts, n, m, voxelsize, n_max, ray_start, ray_dir, points, children,
                    idx, min_depth, max_depth, hits, err, workspace, stream);
}

int nsvf_ball_intersect(int b, int b_pts, int n, int m, float radius, int n_max,
                        const float *ray_start, const float *ray_dir, const float *points,
                        int32_t *idx, float *min_depth, float *max_depth, void *stream) {
  if (bad_common(b, b_pts, n, m, n_max, ray_start, ray_dir, points)) return NSVF_ERR_INVALID;
  int64_t rays = (int64_t)b * m;
  if (rays == 0) return NSVF_OK;
  if (!idx || !min_depth || !max_depth) return NSVF_ERR_INVALID;
  ball_kernel<<<nsvf_grid(rays, kRayBlock), kRayBlock, 0, (cudaStream_t)stream>>>(
      rays, m, b_pts, n, radius, n_max, ray_start, ray_dir, points, idx, min_depth, max_depth);
  return nsvf_launch_status();
}

}  // extern "C"
