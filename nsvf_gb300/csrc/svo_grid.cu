// Sparse-voxel-octree intersection in leaf-grid form: the same sorted hit
// lists as the depth-first traversal (nsvf_svo_intersect_sorted), bit for
// bit, from a sweep along the ray over the grid of leaf voxels.
//
// What the depth-first search computes (fairnr/clib/src/intersect_gpu.cu:
// 170-237, then the encoder's stable depth sort, fairnr/modules/encoder.py:
// 518-524): the leaves whose slab test hits and whose every ancestor's slab
// test hits, the first n_max of them in visiting order (children 7..0), then
// ordered by (min_depth, visiting order).
//
// The leaf-grid form replaces the tree walk by three facts checked once per
// octree on the host (nsvf_svo_grid_build):
//
// 1. Leaves sit on a grid of cells: along each axis, every leaf with grid
//    index i has the same FP32 centre coordinate tab[i], and tab increases
//    with i. A leaf's slab test then splits per axis: along axis a the ray is
//    inside cell i for t in [E_a(i), F_a(i)], with exactly the products the
//    slab test takes, and the leaf (i, j, k) is hit iff
//    max(0, E_x(i), E_y(j), E_z(k)) <= min(1e5, F_x(i), F_y(j), F_z(k)).
//    In travel order along an axis both E and F are non-decreasing (rounding
//    is monotone), so at each t the cells "active" on an axis form a range.
// 2. Ancestors: where every ancestor's FP32 faces (c - h, c + h) enclose the
//    leaf's, a leaf hit implies every ancestor hit (the slab arithmetic is
//    monotone in the face coordinate). Leaves without that property are
//    flagged, and their ancestors' slab tests run explicitly on a hit.
// 3. Order: each leaf's rank in the depth-first visiting order is stored, to
//    order hits with equal min_depth.
//
// The sweep (one thread per ray) processes the cell-entry events of the
// three axes in t order. At an event t, the cells entered at t are new; every
// hit triple with a new member is "born" at t, which is exactly its
// min_depth. Triples are produced in non-decreasing min_depth, each once;
// equal-t triples are ordered by visiting rank. A 4x4x4 brick bitmap with
// prefix counts maps an occupied cell to its leaf. Steps per ray are the grid
// cells the ray crosses (44 on average on the c2 frame), against the
// hundreds of node expansions of the tree walk.
//
// Rays with more than n_max hits (the search stops after the first n_max
// leaves in visiting order) are listed for an overflow pass: a warp per ray
// sweeps it again keeping every hit, and keeps the n_max smallest ranks.
//
// Rays the sweep does not take go to the depth-first kernel, through a list:
// rays with a zero direction component (the slab test's non-finite branch)
// and rays with a hit beyond depth 10000 (the sort puts those after the
// misses).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

int nsvf_svo_sorted_list_launch(int64_t rays, int64_t cap, int n, int n_max,
                                const float *ray_start, const float *ray_dir, const void *packed,
                                const int32_t *ray_list, const int32_t *n_list, int32_t *idx,
                                float *min_depth, float *max_depth, uint8_t *hits, int32_t *err,
                                cudaStream_t stream);

namespace {

constexpr int32_t kGridMagic = 0x3147534e;   // "NSG1"
constexpr int kGridMaxAxis = 1 << 16;
constexpr int64_t kGridMaxBricks = (int64_t)1 << 27;
constexpr int kGridMaxLevels = 16;            // the depth-first kernel's stack levels

// Blob layout: header, per-axis centre tables (x, y, z), bricks (occupancy
// bits of 4x4x4 cells + exclusive prefix count of leaves), leaves in brick
// order (node id, visiting rank | flag << 31), visiting rank per node,
// parent per node. Every section starts on a 16-byte boundary.
struct GridHeader {
  int32_t magic;
  int32_t n[3];
  int32_t nb[3];
  int32_t n_leaves;
  int32_t n_nodes;
  int32_t n_flagged;
  float hv;
  int32_t pad[5];
};
static_assert(sizeof(GridHeader) == 64, "64-byte header");

struct GridLayout {
  int64_t tab, brick, leaf, rank, parent, bytes;
};

__host__ __device__ inline int64_t al16(int64_t x) { return (x + 15) & ~(int64_t)15; }

__host__ __device__ inline GridLayout grid_layout(const int32_t n[3], const int32_t nb[3],
                                                  int32_t n_leaves, int32_t n_nodes) {
  GridLayout L;
  L.tab = (int64_t)sizeof(GridHeader);
  L.brick = al16(L.tab + 4 * ((int64_t)n[0] + n[1] + n[2]));
  L.leaf = L.brick + 16 * (int64_t)nb[0] * nb[1] * nb[2];
  L.rank = al16(L.leaf + 8 * (int64_t)n_leaves);
  L.parent = al16(L.rank + 4 * (int64_t)n_nodes);
  L.bytes = al16(L.parent + 4 * (int64_t)n_nodes);
  return L;
}

// ------------------------------------------------------------ host build --

struct GridPlan {
  GridHeader h;
  std::vector<float> tab[3];
  std::vector<uint64_t> bits;
  std::vector<int32_t> prefix;
  std::vector<int32_t> leaf_id, leaf_rank;
  std::vector<int32_t> rank, parent;
};

// Analyses an octree: NSVF_OK and a plan, NSVF_ERR_OCTREE when the tree is
// not in leaf-grid form (the caller then uses the depth-first kernel, which
// also reports malformed trees).
int grid_plan(int n, float voxelsize, const float *P, const int32_t *C, GridPlan &G) {
  if (n < 1 || !P || !C || !(voxelsize > 0.0f)) return NSVF_ERR_INVALID;
  const float hv = voxelsize * 0.5f;
  G.rank.assign(n, -1);
  G.parent.assign(n, -1);
  std::vector<uint8_t> flag(n, 0);
  std::vector<int32_t> leaves;
  struct Item {
    int32_t k, depth;
    float lo[3], hi[3];   // tightest ancestor faces
  };
  std::vector<Item> stack;
  Item root;
  root.k = n - 1;
  root.depth = 0;
  for (int a = 0; a < 3; ++a) {
    root.lo[a] = -INFINITY;
    root.hi[a] = INFINITY;
  }
  stack.push_back(root);
  int32_t visited = 0;
  while (!stack.empty()) {
    Item it = stack.back();
    stack.pop_back();
    const int32_t k = it.k;
    if (G.rank[k] >= 0 || it.depth >= kGridMaxLevels) return NSVF_ERR_OCTREE;
    G.rank[k] = visited++;
    const int32_t size = C[(int64_t)k * 9 + 8];
    if (size < 1) return NSVF_ERR_OCTREE;
    const float h = hv * (float)size;     // as the packed octree computes it
    float flo[3], fhi[3];
    bool inside = true;
    for (int a = 0; a < 3; ++a) {
      const float c = P[(int64_t)k * 3 + a];
      if (!std::isfinite(c)) return NSVF_ERR_OCTREE;
      flo[a] = c - h;
      fhi[a] = c + h;
      if (flo[a] < it.lo[a] || fhi[a] > it.hi[a]) inside = false;
    }
    if (size == 1) {
      flag[k] = !inside;
      leaves.push_back(k);
      continue;
    }
    for (int u = 0; u < 8; ++u) {
      const int32_t ch = C[(int64_t)k * 9 + u];
      if (ch >= n) return NSVF_ERR_OCTREE;
      if (ch > -1) {
        Item c;
        c.k = ch;
        c.depth = it.depth + 1;
        for (int a = 0; a < 3; ++a) {
          c.lo[a] = std::max(it.lo[a], flo[a]);
          c.hi[a] = std::min(it.hi[a], fhi[a]);
        }
        G.parent[ch] = k;
        stack.push_back(c);
      }
    }
  }
  if (leaves.empty()) return NSVF_ERR_OCTREE;
  const size_t L = leaves.size();
  std::vector<int32_t> cell[3];
  for (int a = 0; a < 3; ++a) {
    double mn = INFINITY, mx = -INFINITY;
    for (int32_t k : leaves) {
      mn = std::min(mn, (double)P[(int64_t)k * 3 + a]);
      mx = std::max(mx, (double)P[(int64_t)k * 3 + a]);
    }
    const double cells = std::floor((mx - mn) / (double)voxelsize + 0.5) + 1.0;
    if (!(cells >= 1.0 && cells <= (double)kGridMaxAxis)) return NSVF_ERR_OCTREE;
    const int32_t na = (int32_t)cells;
    std::vector<float> &t = G.tab[a];
    t.assign(na, NAN);
    cell[a].resize(L);
    for (size_t q = 0; q < L; ++q) {
      const float c = P[(int64_t)leaves[q] * 3 + a];
      const int64_t i = (int64_t)std::floor(((double)c - mn) / (double)voxelsize + 0.5);
      if (i < 0 || i >= na) return NSVF_ERR_OCTREE;
      if (std::isnan(t[i])) t[i] = c;
      else if (t[i] != c) return NSVF_ERR_OCTREE;   // two centres on one grid line
      cell[a][q] = (int32_t)i;
    }
    // grid lines without a leaf: any non-decreasing value keeps the sweep
    // exact (no leaf sits on them)
    float prev = -INFINITY;
    for (int32_t i = 0; i < na; ++i) {
      if (std::isnan(t[i])) t[i] = std::max(prev, (float)(mn + (double)i * (double)voxelsize));
      else if (!(t[i] > prev)) return NSVF_ERR_OCTREE;
      prev = t[i];
    }
    G.h.n[a] = na;
    G.h.nb[a] = (na + 3) / 4;
  }
  const int64_t nbricks = (int64_t)G.h.nb[0] * G.h.nb[1] * G.h.nb[2];
  if (nbricks > kGridMaxBricks) return NSVF_ERR_OCTREE;
  G.bits.assign(nbricks, 0);
  auto brick_of = [&](size_t q, int64_t &w, int &b) {
    const int32_t i = cell[0][q], j = cell[1][q], k = cell[2][q];
    w = ((int64_t)(k >> 2) * G.h.nb[1] + (j >> 2)) * G.h.nb[0] + (i >> 2);
    b = ((k & 3) * 4 + (j & 3)) * 4 + (i & 3);
  };
  for (size_t q = 0; q < L; ++q) {
    int64_t w;
    int b;
    brick_of(q, w, b);
    if ((G.bits[w] >> b) & 1u) return NSVF_ERR_OCTREE;   // two leaves in one cell
    G.bits[w] |= (uint64_t)1 << b;
  }
  G.prefix.assign(nbricks, 0);
  int64_t acc = 0;
  for (int64_t w = 0; w < nbricks; ++w) {
    G.prefix[w] = (int32_t)acc;
    acc += __builtin_popcountll(G.bits[w]);
  }
  G.leaf_id.assign(L, -1);
  G.leaf_rank.assign(L, 0);
  int32_t n_flagged = 0;
  for (size_t q = 0; q < L; ++q) {
    int64_t w;
    int b;
    brick_of(q, w, b);
    const int64_t rk = G.prefix[w] + __builtin_popcountll(G.bits[w] & (((uint64_t)1 << b) - 1));
    const int32_t k = leaves[q];
    G.leaf_id[rk] = k;
    G.leaf_rank[rk] = G.rank[k] | (flag[k] ? (int32_t)0x80000000u : 0);
    n_flagged += flag[k];
  }
  G.h.magic = kGridMagic;
  G.h.n_leaves = (int32_t)L;
  G.h.n_nodes = n;
  G.h.n_flagged = n_flagged;
  G.h.hv = hv;
  for (int q = 0; q < 5; ++q) G.h.pad[q] = 0;
  return NSVF_OK;
}

// ----------------------------------------------------------- the sweep ----

constexpr int kGridBlock = 128;

// The grid as the kernel sees it: pointers into the device blob and its
// dimensions, passed by value (kernel parameters live in the constant bank,
// not in per-thread registers).
struct GridView {
  const float *tab[3];            // grid-line centres per axis
  const ulonglong2 *bricks;       // (occupancy bits, prefix count)
  const int2 *leaf;               // (node id, visiting rank | flag << 31)
  const int32_t *rank_of;         // visiting rank per node
  const int32_t *parent;          // parent per node
  const float *points;            // octree node centres [n, 3]
  const int32_t *children;        // [n, 9]
  int32_t n[3], nb[3];
  float hv;
};

// Per ray: origin, reciprocal direction, and the signed half size (the sign
// of the direction: travel order along the axis).
struct Sweep {
  float o[3], inv[3], sh[3];
};

// Entry (clamped at 0, as the slab test's running max) and exit of the ray
// along axis a through the cell at travel position u.
__device__ __forceinline__ float cell_centre(const GridView &G, const Sweep &S, int a, int u) {
  return __ldg(G.tab[a] + (S.sh[a] > 0.0f ? u : G.n[a] - 1 - u));
}
__device__ __forceinline__ float entry_t(const GridView &G, const Sweep &S, int a, int u) {
  const float c = cell_centre(G, S, a, u);
  const float l = __fmul_rn(__fsub_rn(__fsub_rn(c, S.sh[a]), S.o[a]), S.inv[a]);
  return fmaxf(0.0f, __fadd_rn(l, 0.0f));
}
__device__ __forceinline__ float exit_t(const GridView &G, const Sweep &S, int a, int u) {
  const float c = cell_centre(G, S, a, u);
  return __fmul_rn(__fsub_rn(__fadd_rn(c, S.sh[a]), S.o[a]), S.inv[a]);
}

// The rare paths of the sweep (inlined: as calls they cost 40 % more time).
// Every ancestor of `leaf` passes its slab test (the depth-first kernel's
// test, on the ancestor's box).
__device__ __forceinline__ bool ancestors_hit(const GridView G, float ox, float oy, float oz,
                                           float ix, float iy, float iz, int32_t leaf) {
  const float sx = ix >= 0.0f ? 1.0f : -1.0f, sy = iy >= 0.0f ? 1.0f : -1.0f,
              sz = iz >= 0.0f ? 1.0f : -1.0f;
  int p = __ldg(G.parent + leaf);
  for (int lv = 0; lv < kGridMaxLevels && p >= 0; ++lv) {
    const float hp = fabsf(__fmul_rn(G.hv, (float)__ldg(G.children + (int64_t)p * 9 + 8)));
    float a0, a1;
    if (!nsvf_slab_fast(ox, oy, oz, ix, iy, iz, sx, sy, sz, __ldg(G.points + (int64_t)p * 3 + 0),
                        __ldg(G.points + (int64_t)p * 3 + 1),
                        __ldg(G.points + (int64_t)p * 3 + 2), hp, a0, a1))
      return false;
    p = __ldg(G.parent + p);
  }
  return true;
}

// What a sweep ended with.
constexpr int kSweepDone = 0;     // every hit emitted
constexpr int kSweepList = 1;     // left to the depth-first kernel (a zero direction component,
                                  // or a hit beyond depth 10000)
constexpr int kSweepStopped = 2;  // the emitter stopped it

// The sweep of ray r across the leaf grid: emit(leaf entry, min_depth,
// max_depth) for every hit, in non-decreasing min_depth (hits with equal
// min_depth in any order); emit returns false to stop the sweep.
template <class Emit>
__device__ __forceinline__ int sweep_ray(int64_t r, const GridView &G,
                                         const float *__restrict__ ray_start,
                                         const float *__restrict__ ray_dir, Emit &emit) {
  Sweep S;
  bool fast = true;
  float dir[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    S.o[a] = ray_start[r * 3 + a];
    dir[a] = ray_dir[r * 3 + a];
    S.inv[a] = nsvf_rcp(dir[a]);
    fast = fast && isfinite(S.inv[a]);
    S.sh[a] = S.inv[a] >= 0.0f ? G.hv : -G.hv;
  }
  if (!fast) return kSweepList;
  // the first time inside the grid's slab on every axis, and the cells active
  // then: the first cell (in travel order) not yet left, and the first not yet
  // entered
  float t = 0.0f;
#pragma unroll
  for (int a = 0; a < 3; ++a) t = fmaxf(t, entry_t(G, S, a, 0));
  bool dead = !(t <= 100000.0f);
#pragma unroll
  for (int a = 0; a < 3; ++a) dead = dead || exit_t(G, S, a, G.n[a] - 1) < t;
  if (dead) return kSweepDone;
  int old[3], nxt[3], ns[3];
  float f_old[3], e_nxt[3], f_new[3];   // exits of the first and last active cells
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    // estimate, then correct with the exact exits
    const float c0 = __ldg(G.tab[a]);
    const float x = dir[a] * t + S.o[a];
    float fi = floorf((x - (c0 - G.hv)) / (2.0f * G.hv));
    fi = fminf(fmaxf(fi, 0.0f), (float)(G.n[a] - 1));
    int u = S.sh[a] > 0.0f ? (int)fi : G.n[a] - 1 - (int)fi;
    while (u > 0 && exit_t(G, S, a, u - 1) >= t) --u;
    while (exit_t(G, S, a, u) < t) ++u;            // ends: the last cell's exit >= t
    old[a] = u;
    f_old[a] = exit_t(G, S, a, u);
    int v = u;
    float e = entry_t(G, S, a, v);
    while (e <= t) {
      ++v;
      if (v >= G.n[a]) { e = INFINITY; break; }
      e = entry_t(G, S, a, v);
    }
    nxt[a] = v;
    e_nxt[a] = e;
    f_new[a] = v > u ? exit_t(G, S, a, v - 1) : f_old[a];
    ns[a] = u;                                     // the first event: every active cell is new
  }
  int64_t cached = -1;
  ulonglong2 brick = make_ulonglong2(0, 0);
  int status = kSweepDone;
  // Visits the cell at travel positions (ux, uy, uz), born at t, with the
  // exits fx, fy, fz: emits its leaf if there is one.
  auto visit = [&](int ux, int uy, int uz, float fx, float fy, float fz) {
    const int gi = S.sh[0] > 0.0f ? ux : G.n[0] - 1 - ux;
    const int gj = S.sh[1] > 0.0f ? uy : G.n[1] - 1 - uy;
    const int gk = S.sh[2] > 0.0f ? uz : G.n[2] - 1 - uz;
    const int64_t w = ((int64_t)(gk >> 2) * G.nb[1] + (gj >> 2)) * G.nb[0] + (gi >> 2);
    const int bit = ((gk & 3) * 4 + (gj & 3)) * 4 + (gi & 3);
    if (w != cached) {
      brick = __ldg(G.bricks + w);
      cached = w;
    }
    if (!((brick.x >> bit) & 1ull)) return;
    const int64_t rk = (int64_t)brick.y + __popcll(brick.x & ((1ull << bit) - 1ull));
    const int2 lf = __ldg(G.leaf + rk);
    // a flagged leaf: its ancestors' faces do not all enclose its own
    if (lf.y < 0 && !ancestors_hit(G, S.o[0], S.o[1], S.o[2], S.inv[0], S.inv[1], S.inv[2], lf.x))
      return;
    if (t > NSVF_MAX_DEPTH_F) {
      status = kSweepList;
      return;
    }
    float hi = 100000.0f;
    hi = (fx < hi) ? fx : hi;
    hi = (fy < hi) ? fy : hi;
    hi = (fz < hi) ? fz : hi;
    if (!emit(lf, t, hi)) status = kSweepStopped;
  };
  // each event enters at least one cell (a skip enters the cells at t_j)
  const int64_t max_events = (int64_t)G.n[0] + G.n[1] + G.n[2] + 2;
  for (int64_t ev = 0; !dead && status == kSweepDone && ev < max_events; ++ev) {
    if (old[0] < nxt[0] && old[1] < nxt[1] && old[2] < nxt[2]) {
      // The common event: one axis enters one cell and the other two have
      // one active cell each: one new triple. (On a dyadic grid a cell's
      // exit equals the next cell's entry, so the entering axis's previous
      // cell is still active at t; its triples were born earlier.)
      const int e0 = nxt[0] - ns[0], e1 = nxt[1] - ns[1], e2 = nxt[2] - ns[2];
      const int w0 = nxt[0] - old[0], w1 = nxt[1] - old[1], w2 = nxt[2] - old[2];
      const bool one = (e0 + e1 + e2 == 1) && ((e0 == 1) ? (w1 == 1 && w2 == 1)
                                               : (e1 == 1) ? (w0 == 1 && w2 == 1)
                                                           : (w0 == 1 && w1 == 1));
      if (one) {
        visit(e0 ? nxt[0] - 1 : old[0], e1 ? nxt[1] - 1 : old[1], e2 ? nxt[2] - 1 : old[2],
              e0 ? f_new[0] : f_old[0], e1 ? f_new[1] : f_old[1], e2 ? f_new[2] : f_old[2]);
      } else {
        for (int ux = old[0]; ux < nxt[0] && status == kSweepDone; ++ux) {
          const float fx = exit_t(G, S, 0, ux);
          for (int uy = old[1]; uy < nxt[1] && status == kSweepDone; ++uy) {
            const float fy = exit_t(G, S, 1, uy);
            for (int uz = old[2]; uz < nxt[2] && status == kSweepDone; ++uz) {
              if (ux < ns[0] && uy < ns[1] && uz < ns[2]) continue;   // born earlier
              visit(ux, uy, uz, fx, fy, exit_t(G, S, 2, uz));
            }
          }
        }
      }
    }
    if (status != kSweepDone) break;
    // Brick skip. After t, an axis's cells that can still form triples are
    // the active ones with exit > t and the ones not yet entered. When
    // that is one cell per axis (c) and c's 4x4x4 brick is empty, every
    // triple born before t_j -- the first entry, on any axis, of a cell
    // past the brick -- lies in the brick: those events are taken
    // silently and the sweep resumes at the event t_j.
    float tn = INFINITY;
    bool skip = true;
    int c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const int wdt = nxt[a] - old[a];
      c[a] = (wdt == 1) ? old[a] : old[a] + 1;
      skip = skip && (wdt == 1 || (wdt == 2 && f_old[a] <= t));
    }
    if (skip) {
      const int gi = S.sh[0] > 0.0f ? c[0] : G.n[0] - 1 - c[0];
      const int gj = S.sh[1] > 0.0f ? c[1] : G.n[1] - 1 - c[1];
      const int gk = S.sh[2] > 0.0f ? c[2] : G.n[2] - 1 - c[2];
      const int64_t w = ((int64_t)(gk >> 2) * G.nb[1] + (gj >> 2)) * G.nb[0] + (gi >> 2);
      if (w != cached) {
        brick = __ldg(G.bricks + w);
        cached = w;
      }
      skip = brick.x == 0ull;
      if (skip) {
        const int g3[3] = {gi, gj, gk};
        int lim[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const int rem = S.sh[a] > 0.0f ? 4 - (g3[a] & 3) : (g3[a] & 3) + 1;
          lim[a] = min(G.n[a], c[a] + rem);
          if (lim[a] < G.n[a]) tn = fminf(tn, entry_t(G, S, a, lim[a]));
        }
        if (!(tn <= 100000.0f)) break;          // nothing past this empty brick
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          while (nxt[a] < lim[a] && e_nxt[a] < tn) {
            f_new[a] = exit_t(G, S, a, nxt[a]);
            if (old[a] == nxt[a]) f_old[a] = f_new[a];
            ++nxt[a];
            e_nxt[a] = nxt[a] < G.n[a] ? entry_t(G, S, a, nxt[a]) : INFINITY;
          }
        }
      }
    }
    // the next entry event
    if (!skip) {
      tn = fminf(e_nxt[0], fminf(e_nxt[1], e_nxt[2]));
      if (!(tn <= 100000.0f)) break;
    }
    t = tn;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      while (old[a] < nxt[a] && f_old[a] < t) {
        ++old[a];
        f_old[a] = old[a] == nxt[a] - 1 ? f_new[a]
                   : (old[a] < G.n[a] ? exit_t(G, S, a, old[a]) : 0.0f);
      }
      dead = dead || old[a] >= G.n[a];
      ns[a] = nxt[a];
      while (e_nxt[a] == t) {
        f_new[a] = exit_t(G, S, a, nxt[a]);
        if (old[a] == nxt[a]) f_old[a] = f_new[a];
        ++nxt[a];
        e_nxt[a] = nxt[a] < G.n[a] ? entry_t(G, S, a, nxt[a]) : INFINITY;
      }
    }
  }
  return status;
}

// A hit past a full row, kept for the overflow pass.
struct OverHit {
  uint32_t lo_bits;  // min_depth's bits (>= +0, so they order like the value)
  float hi;
  int32_t id, rank;
};

// Hits past n_max that a ray's overflow block holds; a ray with more goes to
// the depth-first kernel.
constexpr int kOverExtra = 64;

// Emits hits into a ray's row, in (min_depth, visiting rank) order: hits come
// in non-decreasing min_depth, and one with the same min_depth as the row's
// last slots is placed among them by rank. Hits past n_max go, in order, to
// an overflow block reserved for the ray (over slot q); when there is no
// block left or the ray fills it, the sweep stops and the ray goes to the
// depth-first kernel.
struct RowEmit {
  int32_t *I;
  float *LO, *HI;
  const int32_t *rank_of;
  int n_max, cnt;
  float last_lo;                 // min_depth of the row's last slot
  int32_t *n_over;
  OverHit *scratch;
  int over_cap, q, e;
  __device__ __forceinline__ bool operator()(int2 lf, float lo, float hi) {
    if (cnt >= n_max) {
      if (q < 0) {
        q = atomicAdd(n_over, 1);
        if (q >= over_cap) return false;
      }
      if (e >= kOverExtra) return false;
      scratch[(int64_t)q * kOverExtra + e] = OverHit{__float_as_uint(lo), hi, lf.x, lf.y & 0x7fffffff};
      ++e;
      return true;
    }
    int pos = cnt;
    if (cnt > 0 && last_lo == lo) {
      const int32_t my = lf.y & 0x7fffffff;
      while (pos > 0 && LO[pos - 1] == lo && __ldg(rank_of + I[pos - 1]) > my) {
        I[pos] = I[pos - 1];
        LO[pos] = LO[pos - 1];
        HI[pos] = HI[pos - 1];
        --pos;
      }
    }
    I[pos] = lf.x;
    LO[pos] = lo;
    HI[pos] = hi;
    ++cnt;
    last_lo = lo;
    return true;
  }
};

// (No minimum of resident blocks: capping the registers spills and was
// slower on the c2 frame.)
__global__ void __launch_bounds__(kGridBlock) svo_grid_kernel(
    int64_t rays, int n_max, const float *__restrict__ ray_start,
    const float *__restrict__ ray_dir, const GridView G, int32_t *__restrict__ idx,
    float *__restrict__ min_depth, float *__restrict__ max_depth, uint8_t *__restrict__ hits,
    int32_t *__restrict__ list, int32_t *__restrict__ n_list, int32_t *__restrict__ over,
    int32_t *__restrict__ over_cnt, int32_t *__restrict__ n_over, OverHit *__restrict__ scratch,
    int over_cap, unsigned long long *__restrict__ next_ray, bool pad_rows) {
  // Persistent warps: each warp takes the next 32 rays from a global
  // counter until there are none left, so the SMs stay full to the end of
  // the frame (rays differ a lot in length: fixed blocks left the SMs active
  // 57 % of the time, with 7 of 20 possible warps resident on average). A
  // pool of rays per lane (a lane refilling once half its warp is idle) was
  // slower: 0.81 against 0.61 ms on the c2 frame.
  const int lane = threadIdx.x & 31;
  const unsigned full = 0xffffffffu;
  for (;;) {
    unsigned long long base0 = 0;
    if (lane == 0) base0 = atomicAdd(next_ray, 32ull);
    const int64_t base = (int64_t)__shfl_sync(full, base0, 0);
    if (base >= rays) break;
    const int64_t r = base + lane;
    const bool live = r < rays;
    const int64_t rr = live ? r : 0;
    RowEmit em{idx + rr * n_max, min_depth + rr * n_max, max_depth + rr * n_max, G.rank_of,
               n_max, 0, -1.0f, n_over, scratch, over_cap, -1, 0};
    const int st = live ? sweep_ray(rr, G, ray_start, ray_dir, em) : kSweepDone;
    if (em.q >= 0 && em.q < over_cap) {
      // an overflow ray: the overflow pass writes its row (or skips slot q
      // when the ray went to the depth-first kernel)
      over[em.q] = st == kSweepDone ? (int32_t)r : -1;
      over_cnt[em.q] = em.e;
    }
    if (st != kSweepDone) {
      list[atomicAdd(n_list, 1)] = (int32_t)r;
    } else if (live && em.q < 0) {
      hits[r] = em.cnt > 0;
    }
    if (!pad_rows) {
      // rows end at their first -1: a hit ray's row gets one after its last
      // hit (when it has room), a missed ray's row is not written
      if (live && st == kSweepDone && em.q < 0 && em.cnt > 0 && em.cnt < n_max)
        idx[r * n_max + em.cnt] = -1;
      continue;
    }
    // pad the rows (misses: id -1, depths 10000), a warp per row
    const bool pad = live && st == kSweepDone && em.q < 0;
    for (int q = 0; q < 32; ++q) {
      const int cq = __shfl_sync(full, em.cnt, q);
      if (!__shfl_sync(full, (int)pad, q)) continue;
      const int64_t rq = base + q;
      for (int l = cq + lane; l < n_max; l += 32) {
        idx[rq * n_max + l] = -1;
        min_depth[rq * n_max + l] = NSVF_MAX_DEPTH_F;
        max_depth[rq * n_max + l] = NSVF_MAX_DEPTH_F;
      }
    }
  }
}

// Rays with more than n_max hits. The search keeps the first n_max leaves in
// visiting order, then the encoder sorts them by (min_depth, visiting order).
// The sweep wrote such a ray's first n_max hits to its row and the rest to
// its overflow block; a warp per ray gathers both into shared memory, sorts
// them by visiting rank, keeps the first n_max and sorts those by
// (min_depth, rank). (Keeping the n_max smallest ranks in the row during the
// sweep cost a rescan of the row through L2 per replacement, up to 2x the
// sweep's time on views with many such rays; sweeping such rays again in a
// second pass, one lane per ray, took 0.15 ms on the c2 frame.)
constexpr int kOverWarps = 4;
constexpr int kOverMax = 256;     // n_max (<= 128) + kOverExtra, rounded up

// Bitonic sort of buf[0, P) (P a power of two) by key(), ascending, by the
// 32 lanes of a warp.
template <class Key>
__device__ __forceinline__ void warp_bitonic(OverHit *buf, int P, int lane, Key key) {
  for (int size = 2; size <= P; size <<= 1) {
    for (int stride = size >> 1; stride > 0; stride >>= 1) {
      for (int i = lane; i < P / 2; i += 32) {
        const int a = 2 * i - (i & (stride - 1)), b = a + stride;
        const bool asc = (a & size) == 0;
        if ((key(buf[a]) > key(buf[b])) == asc) {
          const OverHit x = buf[a];
          buf[a] = buf[b];
          buf[b] = x;
        }
      }
      __syncwarp();
    }
  }
}

__global__ void __launch_bounds__(32 * kOverWarps) svo_grid_overflow_kernel(
    int n_max, const int32_t *__restrict__ rank_of, int32_t *__restrict__ idx,
    float *__restrict__ min_depth, float *__restrict__ max_depth, uint8_t *__restrict__ hits,
    const int32_t *__restrict__ over, const int32_t *__restrict__ over_cnt,
    const int32_t *__restrict__ n_over, const OverHit *__restrict__ scratch, int over_cap) {
  __shared__ OverHit bufs[kOverWarps][kOverMax];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  OverHit *buf = bufs[w];
  const int64_t n0 = *n_over, n = n0 < over_cap ? n0 : over_cap;
  for (int64_t q = (int64_t)blockIdx.x * kOverWarps + w; q < n;
       q += (int64_t)gridDim.x * kOverWarps) {
    const int64_t r = over[q];
    if (r < 0) continue;                     // the ray went to the depth-first kernel
    const int e = over_cnt[q], k = n_max + e;
    int32_t *I = idx + r * n_max;
    float *LO = min_depth + r * n_max, *HI = max_depth + r * n_max;
    for (int j = lane; j < n_max; j += 32)
      buf[j] = OverHit{__float_as_uint(LO[j]), HI[j], I[j], __ldg(rank_of + I[j])};
    for (int j = lane; j < e; j += 32) buf[n_max + j] = scratch[q * kOverExtra + j];
    int P = 1;
    while (P < k) P <<= 1;
    for (int i = k + lane; i < P; i += 32) buf[i] = OverHit{0xffffffffu, 0.0f, -1, 0x7fffffff};
    __syncwarp();
    warp_bitonic(buf, P, lane, [](const OverHit &h) { return h.rank; });
    // the first n_max ranks, by (min_depth, rank)
    int P2 = 1;
    while (P2 < n_max) P2 <<= 1;
    for (int i = n_max + lane; i < P2; i += 32) buf[i] = OverHit{0xffffffffu, 0.0f, -1, 0x7fffffff};
    __syncwarp();
    warp_bitonic(buf, P2, lane, [](const OverHit &h) {
      return ((unsigned long long)h.lo_bits << 32) | (unsigned)h.rank;
    });
    for (int j = lane; j < n_max; j += 32) {
      I[j] = buf[j].id;
      LO[j] = __uint_as_float(buf[j].lo_bits);
      HI[j] = buf[j].hi;
    }
    if (lane == 0) hits[r] = 1;
    __syncwarp();
  }
}

// The lists' lengths and the persistent warps' ray counter start at 0.
__global__ void zero_kernel(int32_t *n_list, int32_t *n_over, unsigned long long *next_ray) {
  *n_list = 0;
  *n_over = 0;
  *next_ray = 0ull;
}

int g_grid_blocks[64] = {0};   // resident blocks of svo_grid_kernel per device (0: not known)

}  // namespace

extern "C" {

int nsvf_svo_grid_build(int n, float voxelsize, const float *points, const int32_t *children,
                        void *grid, int64_t capacity, int64_t *bytes) {
  GridPlan G;
  const int st = grid_plan(n, voxelsize, points, children, G);
  if (st != NSVF_OK) return st;
  const GridLayout L = grid_layout(G.h.n, G.h.nb, G.h.n_leaves, G.h.n_nodes);
  if (bytes) *bytes = L.bytes;
  if (!grid || capacity < L.bytes) return NSVF_ERR_CAPACITY;
  unsigned char *B = static_cast<unsigned char *>(grid);
  std::fill(B, B + L.bytes, (unsigned char)0);
  std::copy(reinterpret_cast<const unsigned char *>(&G.h),
            reinterpret_cast<const unsigned char *>(&G.h) + sizeof(GridHeader), B);
  float *tab = reinterpret_cast<float *>(B + L.tab);
  for (int a = 0; a < 3; ++a) {
    std::copy(G.tab[a].begin(), G.tab[a].end(), tab);
    tab += G.h.n[a];
  }
  uint64_t *br = reinterpret_cast<uint64_t *>(B + L.brick);
  for (size_t w = 0; w < G.bits.size(); ++w) {
    br[2 * w] = G.bits[w];
    br[2 * w + 1] = (uint64_t)(uint32_t)G.prefix[w];
  }
  int32_t *lf = reinterpret_cast<int32_t *>(B + L.leaf);
  for (size_t q = 0; q < G.leaf_id.size(); ++q) {
    lf[2 * q] = G.leaf_id[q];
    lf[2 * q + 1] = G.leaf_rank[q];
  }
  std::copy(G.rank.begin(), G.rank.end(), reinterpret_cast<int32_t *>(B + L.rank));
  std::copy(G.parent.begin(), G.parent.end(), reinterpret_cast<int32_t *>(B + L.parent));
  return NSVF_OK;
}

int nsvf_svo_grid_info(const void *grid_host, int32_t *out) {
  if (!grid_host || !out) return NSVF_ERR_INVALID;
  const GridHeader *h = static_cast<const GridHeader *>(grid_host);
  if (h->magic != kGridMagic) return NSVF_ERR_INVALID;
  out[0] = h->n[0];
  out[1] = h->n[1];
  out[2] = h->n[2];
  out[3] = h->n_leaves;
  out[4] = h->n_flagged;
  out[5] = h->n_nodes;
  return NSVF_OK;
}

// Overflow blocks of a call of `rays` rays: one per ray up to 32,768.
static int64_t grid_over_cap(int64_t rays) { return rays < 32768 ? (rays > 0 ? rays : 0) : 32768; }

int64_t nsvf_svo_grid_list_bytes(int64_t rays) {
  const int64_t R = rays > 0 ? rays : 0, oc = grid_over_cap(R);
  // counters, ray list, overflow slots (ray, hit count), then 16-byte
  // aligned the overflow blocks
  const int64_t blk_off = (16 + 4 * R + 8 * oc + 15) / 16 * 16;
  return blk_off + oc * kOverExtra * (int64_t)sizeof(OverHit);
}

int nsvf_svo_intersect_grid_rows(int64_t rays, int n, float voxelsize, int n_max,
                                 const float *ray_start, const float *ray_dir,
                                 const float *points, const int32_t *children, const void *grid,
                                 const int32_t *info, const void *packed, void *list_ws,
                                 int32_t *idx, float *min_depth, float *max_depth, uint8_t *hits,
                                 int32_t *err, int pad_rows, void *stream) {
  if (!info || info[5] != n || info[0] < 1 || info[1] < 1 || info[2] < 1 || info[3] < 1)
    return NSVF_ERR_INVALID;
  if (rays < 0 || n < 1 || n_max < 1 || !points || !children || !grid || !packed || !list_ws ||
      (((uintptr_t)grid) & 15) || (((uintptr_t)packed) & 15) || (((uintptr_t)list_ws) & 15))
    return NSVF_ERR_INVALID;
  if (rays == 0) return NSVF_OK;
  if (!ray_start || !ray_dir || !idx || !min_depth || !max_depth || !hits || n_max > 128 ||
      rays > 0x7fffffff)
    return NSVF_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  // list workspace: [0, 4) list length, [4, 8) overflow slots taken, [8, 16)
  // ray counter, then the ray list (rays entries), the overflow slots' rays
  // and hit counts (over_cap entries each) and, 16-byte aligned, the
  // overflow blocks (over_cap x kOverExtra hits)
  const int64_t over_cap = grid_over_cap(rays);
  int32_t *n_list = static_cast<int32_t *>(list_ws);
  int32_t *n_over = n_list + 1;
  unsigned long long *next_ray =
      reinterpret_cast<unsigned long long *>(static_cast<unsigned char *>(list_ws) + 8);
  int32_t *list = n_list + 4;
  int32_t *over = list + rays;
  int32_t *over_cnt = over + over_cap;
  const int64_t blk_off = (16 + 4 * rays + 8 * over_cap + 15) / 16 * 16;
  OverHit *scratch = reinterpret_cast<OverHit *>(static_cast<unsigned char *>(list_ws) + blk_off);
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return NSVF_ERR_CUDA;
  if (g_grid_blocks[dev] == 0) {
    int per_sm = 0, sms = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, svo_grid_kernel, kGridBlock, 0) !=
            cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
      return NSVF_ERR_CUDA;
    g_grid_blocks[dev] = (per_sm > 0 ? per_sm : 1) * (sms > 0 ? sms : 1);
  }
  zero_kernel<<<1, 1, 0, s>>>(n_list, n_over, next_ray);
  int st = nsvf_launch_status();
  if (st != NSVF_OK) return st;
  const unsigned char *B = static_cast<const unsigned char *>(grid);
  GridView G;
  int32_t nb[3];
  for (int a = 0; a < 3; ++a) {
    G.n[a] = info[a];
    G.nb[a] = nb[a] = (info[a] + 3) / 4;
  }
  const GridLayout L = grid_layout(G.n, nb, info[3], info[5]);
  G.tab[0] = reinterpret_cast<const float *>(B + L.tab);
  G.tab[1] = G.tab[0] + G.n[0];
  G.tab[2] = G.tab[1] + G.n[1];
  G.bricks = reinterpret_cast<const ulonglong2 *>(B + L.brick);
  G.leaf = reinterpret_cast<const int2 *>(B + L.leaf);
  G.rank_of = reinterpret_cast<const int32_t *>(B + L.rank);
  G.parent = reinterpret_cast<const int32_t *>(B + L.parent);
  G.points = points;
  G.children = children;
  G.hv = voxelsize * 0.5f;
  const int64_t need = (rays + kGridBlock - 1) / kGridBlock;
  const int blocks = (int)(need < g_grid_blocks[dev] ? need : g_grid_blocks[dev]);
  svo_grid_kernel<<<blocks, kGridBlock, 0, s>>>(rays, n_max, ray_start, ray_dir, G, idx,
                                                min_depth, max_depth, hits, list, n_list, over,
                                                over_cnt, n_over, scratch, (int)over_cap,
                                                next_ray, pad_rows != 0);
  st = nsvf_launch_status();
  if (st != NSVF_OK) return st;
  // the overflow rays: their count is on the device; 8 blocks of 4 warps per
  // SM stride over them
  const int64_t over_blocks = (over_cap + kOverWarps - 1) / kOverWarps;
  svo_grid_overflow_kernel<<<(int)(over_blocks < 152 * 8 ? over_blocks : 152 * 8),
                             32 * kOverWarps, 0, s>>>(n_max, G.rank_of, idx, min_depth,
                                                      max_depth, hits, over, over_cnt, n_over,
                                                      scratch, (int)over_cap);
  st = nsvf_launch_status();
  if (st != NSVF_OK) return st;
  return nsvf_svo_sorted_list_launch(rays, rays, n, n_max, ray_start, ray_dir, packed, list,
                                     n_list, idx, min_depth, max_depth, hits, err, s);
}

int nsvf_svo_intersect_grid(int64_t rays, int n, float voxelsize, int n_max,
                            const float *ray_start, const float *ray_dir, const float *points,
                            const int32_t *children, const void *grid, const int32_t *info,
                            const void *packed, void *list_ws, int32_t *idx, float *min_depth,
                            float *max_depth, uint8_t *hits, int32_t *err, void *stream) {
  return nsvf_svo_intersect_grid_rows(rays, n, voxelsize, n_max, ray_start, ray_dir, points,
                                      children, grid, info, packed, list_ws, idx, min_depth,
                                      max_depth, hits, err, 1, stream);
}

}  // extern "C"
