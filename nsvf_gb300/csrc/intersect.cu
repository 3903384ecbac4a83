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
#include <mutex>

#include <type_traits>

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
  const bool fast = isfinite(ix) && isfinite(iy) && isfinite(iz);
  const float sx = ix >= 0.0f ? 1.0f : -1.0f, sy = iy >= 0.0f ? 1.0f : -1.0f,
              sz = iz >= 0.0f ? 1.0f : -1.0f;
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
        const bool hit =
            fast ? nsvf_slab_fast(ox, oy, oz, ix, iy, iz, sx, sy, sz, sc[k * 3], sc[k * 3 + 1],
                                  sc[k * 3 + 2], hv, lo, hi)
                 : nsvf_slab(ox, oy, oz, ix, iy, iz, sc[k * 3], sc[k * 3 + 1], sc[k * 3 + 2], hv,
                             lo, hi);
        if (hit) {
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

// Packed octree, per point set of n nodes: for node k, its 8 children side
// by side -- ids in kids[8k .. 8k + 7] and boxes in cbox[8k .. 8k + 7] --
// and the root's own box at cbox[8n]. A box is (cx, cy, cz, +half) for an internal
// node and (cx, cy, cz, -half) for a leaf (children[8] == 1); absent
// children get a zero box. The boxes of children c and c + 4 (the two that
// one traversal lane tests) are interleaved component by component:
// cbox[8k + 2c] = (cx_c, cx_c+4, cy_c, cy_c+4) and cbox[8k + 2c + 1] =
// (cz_c, cz_c+4, h_c, h_c+4), c = 0..3, so two 16-byte loads give a lane
// both boxes as pairs for the two-lane (f32x2) slab test; the ids likewise,
// kids[8k + 2c] = id_c and kids[8k + 2c + 1] = id_c+4, one 8-byte load. A node's whole
// child set lies in two 128-byte lines.
__device__ __forceinline__ float4 node_box(const float *__restrict__ P,
                                           const int32_t *__restrict__ C, int k, float hv) {
  int size = C[(int64_t)k * 9 + 8];
  float h = __fmul_rn(hv, (float)size);
  return make_float4(P[(int64_t)k * 3 + 0], P[(int64_t)k * 3 + 1], P[(int64_t)k * 3 + 2],
                     size == 1 ? -h : h);
}

__global__ void pack_octree_kernel(int64_t total, int n, float hv, const float *__restrict__ points,
                                   const int32_t *__restrict__ children, float4 *__restrict__ cbox,
                                   int32_t *__restrict__ kids) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;   // (point set, node, child)
  if (t >= total * 8) return;
  const int j = (int)(t & 7);
  const int64_t gk = t >> 3, g = gk / n;
  const int k = (int)(gk - g * n);
  const int32_t *C = children + g * (int64_t)n * 9;
  const float *P = points + g * (int64_t)n * 3;
  float4 *B = cbox + g * ((int64_t)n * 8 + 1);
  int cid = C[(int64_t)k * 9 + j];
  float4 cb = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (cid > -1 && cid < n) cb = node_box(P, C, cid, hv);
  float *Bf = reinterpret_cast<float *>(B + (int64_t)k * 8 + 2 * (j & 3));
  const int e = j >> 2;                 // first or second of the lane's pair
  Bf[0 + e] = cb.x;
  Bf[2 + e] = cb.y;
  Bf[4 + e] = cb.z;
  Bf[6 + e] = cb.w;
  kids[gk * 8 + 2 * (j & 3) + e] = cid;
  if (k == n - 1 && j == 0) B[(int64_t)n * 8] = node_box(P, C, n - 1, hv);
}

constexpr int kSvoLevels = 16;
constexpr int kLanesPerRay = 4;                       // lane j owns children j and j + 4
static_assert(kLanesPerRay == 4, "the packed octree pairs children c and c + 4 for one lane");
constexpr int kRaysPerWarp = 32 / kLanesPerRay;       // 8
constexpr int kRaysPerBlock = kRayBlock / kLanesPerRay;  // 32

// Warp-cooperative depth-first traversal in the reference's visiting order
// (children 7..0 of every hit node, fairnr/clib/src/intersect_gpu.cu:200-235).
//
// A warp walks 8 rays; the 4 lanes of a ray's group each own two child
// slots (lane j: children j and j + 4). Expanding a node = each lane loads
// its two children's ids and boxes and runs their slab tests; ballots give
// the node's 8-bit masks of hit children and hit leaves. The descent stack
// is spread over the group: lane j keeps, for levels j, j + 4, j + 8 and
// j + 12 (one byte each), the mask of hit children not visited yet (and
// which of them are leaves); the child ids of each level sit in shared
// memory. The next node to expand -- the highest unvisited child of the
// deepest non-empty level -- comes from the group's mask of non-empty levels
// (each lane's stack bytes as bits, OR-ed over the group by two xor
// shuffles) and one shuffle from the level's owner lane, the same on all 4
// lanes. The per-ray bookkeeping (ballots, stack, pick) is shared by twice
// as many rays per warp instruction as with one child per lane.
// When every hit child of a node is a leaf -- always the case for trees made
// by build_octree, whose leaves all sit under depth-0 nodes -- the DFS visits
// them consecutively, so the group emits them at once, the lane of child c
// writing at cnt + (number of hit leaves with a higher index). A leaf met on the stack
// (a node with both leaf and internal children) is emitted on its own. The
// emitted order, the n_max cutoff and every (lo, hi) are the reference's.
// Hits go straight into the output row.

// Warp-cooperative stable sort of one row of n_max <= 32*E slots by
// (min_depth, slot); slots >= cnt are the misses (id -1, depth 10000), the
// reference's masked_fill before its sort. Bitonic network over 32*E keys,
// element j at lane j % 32, register j / 32. Unique keys make any sorting
// network stable. Writes the whole row.
template <int E>
__device__ __forceinline__ void warp_sort_row(int32_t *__restrict__ I, float *__restrict__ LO,
                                              float *__restrict__ HI, int n_max, int cnt,
                                              int lane) {
  float k1[E], hv[E];
  int k2[E], id[E];
#pragma unroll
  for (int e = 0; e < E; ++e) {
    int j = e * 32 + lane;
    if (j < cnt) { k1[e] = LO[j]; k2[e] = j; id[e] = I[j]; hv[e] = HI[j]; }
    else if (j < n_max) { k1[e] = NSVF_MAX_DEPTH_F; k2[e] = j; id[e] = -1; hv[e] = NSVF_MAX_DEPTH_F; }
    else { k1[e] = __int_as_float(0x7f800000); k2[e] = j; id[e] = -1; hv[e] = 0.f; }
  }
  constexpr int N = 32 * E;
#pragma unroll
  for (int k = 2; k <= N; k <<= 1) {
#pragma unroll
    for (int s = k >> 1; s > 0; s >>= 1) {
      if (s >= 32) {
        const int r = s / 32;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          int pe = e ^ r;
          if (pe > e) {
            int j = e * 32 + lane;
            bool asc = (j & k) == 0;
            bool gt = (k1[e] > k1[pe]) || (k1[e] == k1[pe] && k2[e] > k2[pe]);
            if (gt == asc) {
              float a = k1[e]; k1[e] = k1[pe]; k1[pe] = a;
              int b = k2[e]; k2[e] = k2[pe]; k2[pe] = b;
              int c = id[e]; id[e] = id[pe]; id[pe] = c;
              float d = hv[e]; hv[e] = hv[pe]; hv[pe] = d;
            }
          }
        }
      } else {
#pragma unroll
        for (int e = 0; e < E; ++e) {
          int j = e * 32 + lane;
          float o1 = __shfl_xor_sync(0xffffffffu, k1[e], s);
          int o2 = __shfl_xor_sync(0xffffffffu, k2[e], s);
          int oi = __shfl_xor_sync(0xffffffffu, id[e], s);
          float oh = __shfl_xor_sync(0xffffffffu, hv[e], s);
          bool asc = (j & k) == 0;
          bool lower = (j & s) == 0;
          bool other_less = (o1 < k1[e]) || (o1 == k1[e] && o2 < k2[e]);
          bool take = (lower == asc) ? other_less : !other_less;
          if (take) { k1[e] = o1; k2[e] = o2; id[e] = oi; hv[e] = oh; }
        }
      }
    }
  }
#pragma unroll
  for (int e = 0; e < E; ++e) {
    int j = e * 32 + lane;
    if (j < n_max) { I[j] = id[e]; LO[j] = k1[e]; HI[j] = hv[e]; }
  }
}

// f32x2 helpers: two FP32 lanes per instruction, each rounded as the
// scalar __fadd_rn / __fsub_rn / __fmul_rn would.
__device__ __forceinline__ uint64_t f2(float lo, float hi) {
  uint64_t d;
  asm("mov.b64 %0, {%1, %2};\n" : "=l"(d) : "f"(lo), "f"(hi));
  return d;
}
__device__ __forceinline__ void f2_split(uint64_t v, float &lo, float &hi) {
  asm("mov.b64 {%0, %1}, %2;\n" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ uint64_t f2_add(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("add.rn.f32x2 %0, %1, %2;\n" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t f2_sub(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("sub.rn.f32x2 %0, %1, %2;\n" : "=l"(d) : "l"(a), "l"(b));
  return d;
}
__device__ __forceinline__ uint64_t f2_mul(uint64_t a, uint64_t b) {
  uint64_t d;
  asm("mul.rn.f32x2 %0, %1, %2;\n" : "=l"(d) : "l"(a), "l"(b));
  return d;
}

// nsvf_slab_fast on two boxes at once, given as pairs of their components
// (c = (c_0, c_1) per axis, h = (|h_0|, |h_1|)): the same operations in the
// same order on each lane, so each result equals nsvf_slab_fast's.
__device__ __forceinline__ void slab_fast_pair(float ox, float oy, float oz, float ix, float iy,
                                               float iz, float sx, float sy, float sz,
                                               uint64_t cx, uint64_t cy, uint64_t cz, uint64_t h,
                                               bool (&hit)[2], float (&t_lo)[2],
                                               float (&t_hi)[2]) {
  float lo[2] = {0.0f, 0.0f}, hi[2] = {100000.0f, 100000.0f};
  const uint64_t zero = 0;
  auto axis = [&](uint64_t c, float s, float o, float inv) {
    const uint64_t sh = f2_mul(f2(s, s), h), oo = f2(o, o), ii = f2(inv, inv);
    const uint64_t l = f2_add(f2_mul(f2_sub(f2_sub(c, sh), oo), ii), zero);
    const uint64_t u = f2_mul(f2_sub(f2_add(c, sh), oo), ii);
    float l0, l1, u0, u1;
    f2_split(l, l0, l1);
    f2_split(u, u0, u1);
    lo[0] = fmaxf(lo[0], l0);
    lo[1] = fmaxf(lo[1], l1);
    hi[0] = (u0 < hi[0]) ? u0 : hi[0];
    hi[1] = (u1 < hi[1]) ? u1 : hi[1];
  };
  axis(cx, sx, ox, ix);
  axis(cy, sy, oy, iy);
  axis(cz, sz, oz, iz);
#pragma unroll
  for (int e = 0; e < 2; ++e) {
    t_lo[e] = lo[e];
    t_hi[e] = hi[e];
    hit[e] = !(lo[e] > hi[e]);
  }
}

template <bool SORTED>
__global__ void __launch_bounds__(kRayBlock) svo_kernel(
    int64_t rays, int m, int b_pts, int n, int n_max, const float *__restrict__ ray_start,
    const float *__restrict__ ray_dir, const float4 *__restrict__ cbox_all,
    const int32_t *__restrict__ kids_all, int32_t *__restrict__ idx, float *__restrict__ min_depth,
    float *__restrict__ max_depth, uint8_t *__restrict__ hits, int32_t *__restrict__ err,
    const int32_t *__restrict__ ray_list, const int32_t *__restrict__ n_list) {
  // per ray and stack level: the expanded node's 8 child ids (lane j writes
  // children j + P c) and the node's id
  __shared__ int s_child[kSvoLevels * kRaysPerBlock * 8];
  __shared__ int s_node[kSvoLevels * kRaysPerBlock];
  const uint32_t full = 0xffffffffu;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int grp = lane / kLanesPerRay, j = lane % kLanesPerRay;  // ray slot, child slots j + P c
  const int g0 = lane - j;                           // the group's first lane
  const uint32_t gshift = (uint32_t)(kLanesPerRay * grp);
  const int slot = warp * kRaysPerWarp + grp;        // ray slot in the block
  // Ray-list mode (ray_list != NULL): slot q of the launch takes ray
  // ray_list[q] for q < *n_list; blocks past the list return at once (the
  // test is the same for the whole block).
  int64_t r = (int64_t)blockIdx.x * kRaysPerBlock + slot;
  bool live = r < rays;
  if (ray_list) {
    const int64_t nl = *n_list;
    if ((int64_t)blockIdx.x * kRaysPerBlock >= nl) return;
    live = r < nl;
    r = live ? (int64_t)ray_list[r] : 0;
  }
  bool bad = false;
  int cnt = 0;

  const int64_t rr = live ? r : 0;
  const int64_t g = (b_pts == 1) ? 0 : rr / m;
  const float4 *CB = cbox_all + g * ((int64_t)n * 8 + 1);
  const int32_t *KD = kids_all + g * (int64_t)n * 8;
  const float ox = ray_start[rr * 3 + 0], oy = ray_start[rr * 3 + 1], oz = ray_start[rr * 3 + 2];
  const float ix = nsvf_rcp(ray_dir[rr * 3 + 0]), iy = nsvf_rcp(ray_dir[rr * 3 + 1]),
              iz = nsvf_rcp(ray_dir[rr * 3 + 2]);
  // the compare/select-light slab test for rays without a zero direction
  // component (the same on the group's lanes)
  const bool fast = isfinite(ix) && isfinite(iy) && isfinite(iz);
  const float sx = ix >= 0.0f ? 1.0f : -1.0f, sy = iy >= 0.0f ? 1.0f : -1.0f,
              sz = iz >= 0.0f ? 1.0f : -1.0f;
  auto slab = [&](float cx, float cy, float cz, float h, float &lo, float &hi) {
    return fast ? nsvf_slab_fast(ox, oy, oz, ix, iy, iz, sx, sy, sz, cx, cy, cz, h, lo, hi)
                : nsvf_slab(ox, oy, oz, ix, iy, iz, cx, cy, cz, h, lo, hi);
  };
  int32_t *I = idx + rr * n_max;
  float *LO = min_depth + rr * n_max, *HI = max_depth + rr * n_max;

  // root
  int level = -1;
  {
    float4 rb = CB[(int64_t)n * 8];
    float lo, hi;
    bool rh = live && slab(rb.x, rb.y, rb.z, fabsf(rb.w), lo, hi);
    if (rh && rb.w < 0.0f) {            // a single-leaf octree
      if (j == 0) { I[0] = n - 1; LO[0] = lo; HI[0] = hi; }
      cnt = 1;
    } else if (rh) {
      level = 0;
    }
  }
  // lane j's share of the stack: byte k holds level j + P k (P lanes per ray)
  constexpr int P = kLanesPerRay, NC = 8 / P, NLV = kSvoLevels / P;
  constexpr uint32_t PM = (1u << P) - 1u;
  using Stack = typename std::conditional<(NLV * 8 > 32), uint64_t, uint32_t>::type;
  Stack stk = 0, stl = 0;               // unvisited hit children; those that are leaves
  int node = n - 1;                      // the node to expand next (valid when `expand`)
  bool expand = level == 0;
  int64_t steps = 0;
  // Every group runs the loop until all groups of the warp are done. All
  // warp-wide operations run on all 32 lanes every iteration; only
  // lane-local work is predicated on `expand` / `pick`. Every value the
  // group steers by (level, cnt, node, top, t, u) is the same on its lanes.
  while (__any_sync(full, expand)) {
    // 1. expand `node`: lane j tests children j + P c
    bool hit[NC];
    float clo[NC], chi[NC], cbw[NC];
    int cid[NC];
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      hit[c] = false;
      clo[c] = chi[c] = cbw[c] = 0.0f;
      cid[c] = -1;
    }
    if (expand) {
      // children j and j + 4: ids, and both boxes as component pairs
      const int2 ids = *reinterpret_cast<const int2 *>(KD + (int64_t)node * 8 + 2 * j);
      const float4 qa = CB[(int64_t)node * 8 + 2 * j], qb = CB[(int64_t)node * 8 + 2 * j + 1];
      bool sh[NC];
      if (fast) {
        slab_fast_pair(ox, oy, oz, ix, iy, iz, sx, sy, sz, f2(qa.x, qa.y), f2(qa.z, qa.w),
                       f2(qb.x, qb.y), f2(fabsf(qb.z), fabsf(qb.w)), sh, clo, chi);
      } else {
        sh[0] = nsvf_slab(ox, oy, oz, ix, iy, iz, qa.x, qa.z, qb.x, fabsf(qb.z), clo[0], chi[0]);
        sh[1] = nsvf_slab(ox, oy, oz, ix, iy, iz, qa.y, qa.w, qb.y, fabsf(qb.w), clo[1], chi[1]);
      }
      cbw[0] = qb.z;
      cbw[1] = qb.w;
      cid[0] = ids.x;
      cid[1] = ids.y;
#pragma unroll
      for (int c = 0; c < NC; ++c) {
        if (cid[c] > -1) {
          if (cid[c] >= n) bad = true;
          else hit[c] = sh[c];
        }
      }
    }
    uint32_t hm = 0, lm = 0;
#pragma unroll
    for (int c = 0; c < NC; ++c) {
      hm |= ((__ballot_sync(full, hit[c]) >> gshift) & PM) << (P * c);
      lm |= ((__ballot_sync(full, hit[c] && cbw[c] < 0.0f) >> gshift) & PM) << (P * c);
    }
    if (expand && ++steps > 8 * (int64_t)n) { bad = true; expand = false; }
    int top = level - 1;                  // deepest stack level that may hold children
    if (expand) {
      if (hm != 0 && hm == lm) {
        // all hit children are leaves: emit them now, highest index first
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const int before = __popc(hm >> (j + P * c + 1));
          if (hit[c] && cnt + before < n_max) {
            I[cnt + before] = cid[c]; LO[cnt + before] = clo[c]; HI[cnt + before] = chi[c];
          }
        }
        cnt = min(n_max, cnt + __popc(hm));
      } else if (hm != 0) {
        const int base = level * kRaysPerBlock + slot;
#pragma unroll
        for (int c = 0; c < NC; ++c) s_child[base * 8 + j + P * c] = cid[c];
        if (j == 0) s_node[base] = node;
        if (j == level % P) {
          const int sh = (level / P) * 8;
          stk = (stk & ~((Stack)0xffu << sh)) | ((Stack)hm << sh);
          stl = (stl & ~((Stack)0xffu << sh)) | ((Stack)lm << sh);
        }
        top = level;
      }
    }
    __syncwarp();                         // s_child / s_node writes -> the group's reads
    // 2. the next node to expand: the highest unvisited child of the deepest
    // non-empty level <= top. A leaf found there is emitted and the pick
    // repeats.
    bool pick = expand && cnt < n_max;
    int next = -1;
    while (__any_sync(full, pick)) {
      // bit l of L: level l (<= top) still has unvisited children. Level
      // P k + j is byte k of lane j: each lane sets bits j + P k for its
      // non-empty bytes, and two xor shuffles OR them over the group.
      static_assert(P == 4 && NLV == 4, "four one-byte levels per lane");
      uint32_t own = 0;
      if (pick && top >= 0) {
        const uint32_t s32 = (uint32_t)stk;
        // the high bit of every non-zero byte
        const uint32_t nzb = (((s32 & 0x7f7f7f7fu) + 0x7f7f7f7fu) | s32) & 0x80808080u;
        // bytes 0..3 (bits 7, 15, 23, 31) to bits 0, 4, 8, 12
        const uint32_t sp = ((nzb >> 7) & 0x1u) | ((nzb >> 11) & 0x10u) | ((nzb >> 15) & 0x100u) |
                            ((nzb >> 19) & 0x1000u);
        own = (sp << j) & ((2u << top) - 1u);  // levels 0..top (top <= 15)
      }
      uint32_t L = own;
      L |= __shfl_xor_sync(full, L, 1);
      L |= __shfl_xor_sync(full, L, 2);
      const int t = (pick && L != 0) ? 31 - __clz(L) : -1;
      uint32_t mine = 0, isleaf = 0;
      int u = 0;
      if (t >= 0 && j == t % P) {
        const int sh = (t / P) * 8;
        mine = (uint32_t)(stk >> sh) & 0xffu;
        u = 31 - __clz(mine);
        isleaf = (uint32_t)(stl >> (sh + u)) & 1u;
        stk &= ~((Stack)1u << (sh + u));
      }
      const int src = g0 + (t >= 0 ? t % P : 0);
      u = __shfl_sync(full, u, src);
      isleaf = __shfl_sync(full, isleaf, src);
      if (pick) {
        if (t < 0) {
          pick = false;                   // the stack is empty: the ray is done
        } else {
          const int base = t * kRaysPerBlock + slot;
          const int ch = s_child[base * 8 + u];
          top = t;
          if (isleaf) {
            if (j == 0) {
              const float *cb =
                  reinterpret_cast<const float *>(CB + (int64_t)s_node[base] * 8 + 2 * (u & 3)) +
                  (u >> 2);
              float a, b2;
              slab(cb[0], cb[2], cb[4], -cb[6], a, b2);
              I[cnt] = ch; LO[cnt] = a; HI[cnt] = b2;
            }
            ++cnt;
            if (cnt >= n_max) pick = false;
          } else if (t + 1 >= kSvoLevels) {
            bad = true;
            pick = false;
          } else {
            next = ch;
            level = t + 1;
            pick = false;
          }
        }
      }
    }
    if (expand) {
      if (next >= 0) node = next;
      else expand = false;
    }
  }
  if (live && SORTED && j == 0) hits[r] = cnt > 0;
  if (bad && err) atomicOr(err, 1);
  __syncwarp();
  // rows: sorted variant sorts (and pads) every row with a hit and pads the
  // empty ones; the raw variant pads with (-1, 0, 0)
  for (int q = 0; q < kRaysPerWarp; ++q) {
    int cq = __shfl_sync(0xffffffffu, cnt, q * kLanesPerRay);
    bool lq = __shfl_sync(0xffffffffu, (int)live, q * kLanesPerRay) != 0;
    const int64_t rq = __shfl_sync(0xffffffffu, (long long)r, q * kLanesPerRay);
    if (!lq) continue;
    int32_t *Iq = idx + rq * n_max;
    float *Lq = min_depth + rq * n_max, *Hq = max_depth + rq * n_max;
    if (SORTED && cq > 0) {
      // A row with at most 32 hits, all at depths <= 10000 (not NaN), sorts
      // as its first 32 slots: the whole row's order puts the same misses
      // (depth 10000, in slot order) after them.
      const bool short_row =
          n_max > 32 && cq <= 32 &&
          __all_sync(0xffffffffu, lane >= cq || Lq[lane] <= NSVF_MAX_DEPTH_F);
      if (n_max <= 32) {
        warp_sort_row<1>(Iq, Lq, Hq, n_max, cq, lane);
      } else if (short_row) {
        warp_sort_row<1>(Iq, Lq, Hq, 32, cq, lane);
        for (int l = 32 + lane; l < n_max; l += 32) {
          Iq[l] = -1; Lq[l] = NSVF_MAX_DEPTH_F; Hq[l] = NSVF_MAX_DEPTH_F;
        }
      } else if (n_max <= 64) {
        warp_sort_row<2>(Iq, Lq, Hq, n_max, cq, lane);
      } else {
        warp_sort_row<4>(Iq, Lq, Hq, n_max, cq, lane);
      }
    } else {
      float pad = SORTED ? NSVF_MAX_DEPTH_F : 0.0f;
      for (int l = cq + lane; l < n_max; l += 32) { Iq[l] = -1; Lq[l] = pad; Hq[l] = pad; }
    }
    __syncwarp();
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

// ------------------------------------------------------------ triangle ----

constexpr int kTriTile = 512;   // faces per shared-memory tile (18 KB)

// The reference's float3 helpers as nvcc contracts them
// (fairnr/clib/include/cutil_math.h:404-413, first product of a sum fused):
// dot -> fma(z, z', fma(x, x', y*y')), cross a*b - c*d -> fma(a, b, -(c*d)).
__device__ __forceinline__ float tri_dot(float ax, float ay, float az, float bx, float by,
                                         float bz) {
  return __fmaf_rn(az, bz, __fmaf_rn(ax, bx, __fmul_rn(ay, by)));
}
__device__ __forceinline__ float tri_cr(float a, float b, float c, float d) {
  return __fmaf_rn(a, b, -__fmul_rn(c, d));
}

// RayTriangleIntersection (fairnr/clib/src/intersect_gpu.cu:238-270):
// Moller-Trumbore with a `blur` margin on the barycentrics; t (> 0 on a hit)
// and (u, v). 1/det is the correctly rounded reciprocal (the reference's
// __fdividef is approximate).
__device__ __forceinline__ float tri_test(float ox, float oy, float oz, float dx, float dy,
                                          float dz, const float *__restrict__ f, float blur,
                                          float &u_out, float &v_out) {
  const float e1x = __fsub_rn(f[3], f[0]), e1y = __fsub_rn(f[4], f[1]), e1z = __fsub_rn(f[5], f[2]);
  const float e2x = __fsub_rn(f[6], f[0]), e2y = __fsub_rn(f[7], f[1]), e2z = __fsub_rn(f[8], f[2]);
  const float vx = __fsub_rn(ox, f[0]), vy = __fsub_rn(oy, f[1]), vz = __fsub_rn(oz, f[2]);
  const float px = tri_cr(dy, e2z, dz, e2y), py = tri_cr(dz, e2x, dx, e2z),
              pz = tri_cr(dx, e2y, dy, e2x);
  const float det = nsvf_rcp(tri_dot(e1x, e1y, e1z, px, py, pz));
  const float u = __fmul_rn(tri_dot(vx, vy, vz, px, py, pz), det);
  const float lo = __fsub_rn(0.0f, blur), hi = __fadd_rn(1.0f, blur);
  if ((u < lo) || (u > hi)) return -1.0f;
  const float qx = tri_cr(vy, e1z, vz, e1y), qy = tri_cr(vz, e1x, vx, e1z),
              qz = tri_cr(vx, e1y, vy, e1x);
  const float v = __fmul_rn(tri_dot(dx, dy, dz, qx, qy, qz), det);
  if ((v < lo) || (v > hi)) return -1.0f;
  const float uv = __fadd_rn(u, v);
  if ((uv < lo) || (uv > hi)) return -1.0f;
  u_out = u;
  v_out = v;
  return __fmul_rn(tri_dot(e2x, e2y, e2z, qx, qy, qz), det);
}

// One thread per ray, faces staged through shared memory in tiles; the
// first n_max hits in face order kept depth-sorted by insertion, then the
// per-hit depth offsets (fairnr/clib/src/intersect_gpu.cu:273-345).
__global__ void __launch_bounds__(kRayBlock) triangle_kernel(
    int b, int b_faces, int n, int m, float cagesize, float blur, int n_max,
    const float *__restrict__ ray_start, const float *__restrict__ ray_dir,
    const float *__restrict__ faces, int32_t *__restrict__ idx, float *__restrict__ depth,
    float *__restrict__ uv) {
  __shared__ float sf[kTriTile * 9];
  const int blocks_per_row = (m + kRayBlock - 1) / kRayBlock;
  const int g = blockIdx.x / blocks_per_row;
  const int j = (blockIdx.x % blocks_per_row) * kRayBlock + threadIdx.x;
  const bool live = j < m;
  const int64_t r = (int64_t)g * m + (live ? j : 0);
  const float *F = faces + (b_faces == 1 ? 0 : (int64_t)g * n * 9);
  float ox = 0, oy = 0, oz = 0, dx = 0, dy = 0, dz = 0;
  if (live) {
    ox = ray_start[r * 3 + 0]; oy = ray_start[r * 3 + 1]; oz = ray_start[r * 3 + 2];
    dx = ray_dir[r * 3 + 0]; dy = ray_dir[r * 3 + 1]; dz = ray_dir[r * 3 + 2];
  }
  int32_t *I = idx + r * n_max;
  float *D = depth + r * n_max * 3, *UV = uv + r * n_max * 2;
  int cnt = 0;
  for (int base = 0; base < n; base += kTriTile) {
    const int tile = min(kTriTile, n - base);
    if (__syncthreads_and(!live || cnt >= n_max)) break;
    for (int t = threadIdx.x; t < tile * 9; t += kRayBlock) sf[t] = F[(int64_t)base * 9 + t];
    __syncthreads();
    if (live) {
      for (int k = 0; k < tile && cnt < n_max; ++k) {
        float u, v;
        float t = tri_test(ox, oy, oz, dx, dy, dz, sf + k * 9, blur, u, v);
        if (!(t > 0.0f)) continue;
        int ki = base + k;
        for (int l = 0; l < cnt; ++l) {
          if (t < D[3 * l]) {
            int ti = I[l]; I[l] = ki; ki = ti;
            float tt = D[3 * l]; D[3 * l] = t; t = tt;
            float tu = UV[2 * l]; UV[2 * l] = u; u = tu;
            float tv = UV[2 * l + 1]; UV[2 * l + 1] = v; v = tv;
          }
        }
        I[cnt] = ki; D[3 * cnt] = t; UV[2 * cnt] = u; UV[2 * cnt + 1] = v;
        ++cnt;
      }
    }
    __syncthreads();
  }
  if (!live) return;
  for (int l = 0; l < cnt; ++l) {
    D[3 * l + 1] = (l == 0) ? -cagesize
                            : -fminf(cagesize, __fmul_rn(0.5f, __fsub_rn(D[3 * l], D[3 * l - 3])));
    D[3 * l + 2] = (l == cnt - 1)
                       ? cagesize
                       : fminf(cagesize, __fmul_rn(0.5f, __fsub_rn(D[3 * l + 3], D[3 * l])));
  }
  for (int l = cnt; l < n_max; ++l) {
    I[l] = -1;
    D[3 * l] = D[3 * l + 1] = D[3 * l + 2] = 0.0f;
    UV[2 * l] = UV[2 * l + 1] = 0.0f;
  }
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

// Packed octree per point set: (8n + 1) boxes of 16 bytes, then (for all
// sets) 8n child ids of 4 bytes.
int64_t nsvf_svo_workspace_bytes(int b_pts, int n) {
  return (int64_t)b_pts * (((int64_t)n * 8 + 1) * (int64_t)sizeof(float4) +
                           (int64_t)n * 8 * (int64_t)sizeof(int32_t));
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
  float4 *cbox = (float4 *)workspace;
  int32_t *kids = (int32_t *)(cbox + (int64_t)b_pts * ((int64_t)n * 8 + 1));
  float hv = voxelsize * 0.5f;
  pack_octree_kernel<<<nsvf_grid(total * 8, 256), 256, 0, s>>>(total, n, hv, points, children,
                                                               cbox, kids);
  nsvf_count_launch();
  int64_t rays = (int64_t)b * m;
  if (rays == 0) return nsvf_launch_status();
  if (sorted)
    svo_kernel<true><<<nsvf_grid(rays, kRaysPerBlock), kRayBlock, 0, s>>>(
        rays, m, b_pts, n, n_max, ray_start, ray_dir, cbox, kids, idx, min_depth, max_depth, hits,
        err, nullptr, nullptr);
  else
    svo_kernel<false><<<nsvf_grid(rays, kRaysPerBlock), kRayBlock, 0, s>>>(
        rays, m, b_pts, n, n_max, ray_start, ray_dir, cbox, kids, idx, min_depth, max_depth, hits,
        err, nullptr, nullptr);
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

int nsvf_svo_pack(int n, float voxelsize, const float *points, const int32_t *children,
                  void *workspace, void *stream) {
  if (n < 1 || !points || !children || !workspace || (((uintptr_t)workspace) & 15))
    return NSVF_ERR_INVALID;
  float4 *cbox = (float4 *)workspace;
  int32_t *kids = (int32_t *)(cbox + ((int64_t)n * 8 + 1));
  pack_octree_kernel<<<nsvf_grid((int64_t)n * 8, 256), 256, 0, (cudaStream_t)stream>>>(
      n, n, voxelsize * 0.5f, points, children, cbox, kids);
  return nsvf_launch_status();
}

}  // extern "C"

// The sorted traversal over a device-side list of rays (one octree, packed
// by nsvf_svo_pack into `packed`): the leaf-grid intersection's fallback for
// the rays it leaves to the depth-first search. The launch covers `cap` list
// slots; blocks past the list's device-side length return at once.
int nsvf_svo_sorted_list_launch(int64_t rays, int64_t cap, int n, int n_max,
                                const float *ray_start, const float *ray_dir, const void *packed,
                                const int32_t *ray_list, const int32_t *n_list, int32_t *idx,
                                float *min_depth, float *max_depth, uint8_t *hits, int32_t *err,
                                cudaStream_t stream) {
  if (cap <= 0) return NSVF_OK;
  const float4 *cbox = (const float4 *)packed;
  const int32_t *kids = (const int32_t *)(cbox + ((int64_t)n * 8 + 1));
  svo_kernel<true><<<nsvf_grid(cap, kRaysPerBlock), kRayBlock, 0, stream>>>(
      rays, (int)(rays > 0x7fffffff ? 0x7fffffff : rays), 1, n, n_max, ray_start, ray_dir, cbox,
      kids, idx, min_depth, max_depth, hits, err, ray_list, n_list);
  return nsvf_launch_status();
}

extern "C" {

// ------------------------------------------------------------------------
// SVO intersection without any device allocation.
//
// For callers that cannot allocate device memory on the call path -- a
// real-time render loop or a host engine that pre-partitions GPU memory and
// hands this library only its own input and output buffers -- the
// packed-octree scratch that nsvf_svo_intersect takes as `workspace` lives
// here in a file-scope device array instead. Its size is fixed:
// NSVF_NOALLOC_MAX_NODES nodes (b_pts * n) at 176 bytes each (160 for the
// packed node, 16 for a point set's root box in the worst case of one node
// per set), 44 MiB, which every GPU that loads this library holds until the
// process exits. Host code only sees a stand-in for the array's name, never
// its device address, so the address is looked up once per device with
// cudaGetSymbolAddress (with that device current) and cached. The cache
// does not survive a device reset: after cudaDeviceReset (or a released and
// re-created primary context) the module may load at another address, and a
// process that resets a device must not call this entry point on it again.
static __device__ __align__(256) unsigned char g_svo_noalloc_scratch[(size_t)NSVF_NOALLOC_MAX_NODES * 176];

static void *noalloc_scratch_for_current_device(int *status) {
  static std::mutex mu;
  static void *addr[256] = {nullptr};
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) {
    *status = NSVF_ERR_CUDA;
    return nullptr;
  }
  std::lock_guard<std::mutex> lock(mu);
  if (!addr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_svo_noalloc_scratch) != cudaSuccess || !p) {
      *status = NSVF_ERR_CUDA;
      return nullptr;
    }
    addr[dev] = p;
  }
  return addr[dev];
}

int nsvf_svo_intersect_noalloc(int b, int b_pts, int n, int m, float voxelsize, int n_max,
                               const float *ray_start, const float *ray_dir, const float *points,
                               const int32_t *children, int32_t *idx, float *min_depth,
                               float *max_depth, int32_t *err, void *stream) {
  if (b_pts < 1 || n < 1 || (int64_t)b_pts * n > (int64_t)NSVF_NOALLOC_MAX_NODES)
    return (b_pts >= 1 && n >= 1) ? NSVF_ERR_CAPACITY : NSVF_ERR_INVALID;
  int status = NSVF_OK;
  void *scratch = noalloc_scratch_for_current_device(&status);
  if (!scratch) return status;
  // the pack kernel rewrites all b_pts * n scratch entries before the
  // traversal reads them, so nothing left by an earlier call is read
  return svo_launch(false, b, b_pts, n, m, voxelsize, n_max, ray_start, ray_dir, points, children,
                    idx, min_depth, max_depth, nullptr, err, scratch, stream);
}

int nsvf_triangle_intersect(int b, int b_faces, int n, int m, float cagesize, float blur,
                            int n_max, const float *ray_start, const float *ray_dir,
                            const float *face_points, int32_t *idx, float *depth, float *uv,
                            void *stream) {
  if (bad_common(b, b_faces, n, m, n_max, ray_start, ray_dir, face_points)) return NSVF_ERR_INVALID;
  if ((int64_t)b * m == 0) return NSVF_OK;
  if (!idx || !depth || !uv) return NSVF_ERR_INVALID;
  int blocks_per_row = (m + kRayBlock - 1) / kRayBlock;
  int64_t grid = (int64_t)b * blocks_per_row;
  if (grid > 0x7fffffff) return NSVF_ERR_INVALID;
  triangle_kernel<<<(int)grid, kRayBlock, 0, (cudaStream_t)stream>>>(
      b, b_faces, n, m, cagesize, blur, n_max, ray_start, ray_dir, face_points, idx, depth, uv);
  return nsvf_launch_status();
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
