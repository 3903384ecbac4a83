// Sample placement inside the hit intervals: inverse-CDF (the sampler NSVF
// uses) and the three-way-merge uniform sampler.
//
// Reference behaviour: fairnr/clib/src/sample_gpu.cu:15-202 and
// fairnr/clib/src/sample.cpp:23-96. FP32 with the reference's operation order;
// `a + b * c` is written as __fmaf_rn where nvcc contracts it in the
// reference build (this file is compiled with -fmad=false so that no other
// contraction happens).
#include "common.cuh"

namespace {

constexpr int kBlock = 128;

__device__ __forceinline__ void warp_max_atomic(int32_t *dst, int v, bool live) {
  unsigned mask = __activemask();
  int x = live ? v : 0;
  for (int o = 16; o > 0; o >>= 1) x = max(x, __shfl_xor_sync(mask, x, o));
  if ((threadIdx.x & 31) == (__ffs(mask) - 1) && dst) atomicMax(dst, x);
}

// Walk of one ray's piecewise-uniform CDF over its hit intervals
// (fairnr/clib/src/sample_gpu.cu:108-202). `emit(id, depth, dist)` receives
// the samples in order and returns false when it has no room (the walk then
// stops and reports overflow). Returns true on overflow.
//   I, lo, hi, pr : this ray's H slots; I0 : the block's first row (tail
//   test); nxt : row whose first id is read when the tail runs past slot H
//   (-1 = none); U : jitter row (NULL = 0.5), noise_cols its width.
template <typename Emit>
__device__ __forceinline__ bool icdf_walk(int H, const int32_t *__restrict__ I,
                                          const int32_t *__restrict__ I0,
                                          const int32_t *__restrict__ pts_all, int64_t nxt,
                                          const float *__restrict__ lo,
                                          const float *__restrict__ hi,
                                          const float *__restrict__ pr, float steps,
                                          const float *__restrict__ U, int noise_cols,
                                          float fixed_step_size, Emit &emit) {
  int bin = 0;
  float cmin = lo[0], cmax = hi[0];
  float cdf_lo = 0.0f, cdf_hi = pr[0];
  float step_size = __double2float_rn(__ddiv_rn(1.0, (double)steps));
  float z_low = cmin;
  int total_steps = (int)ceilf(steps);
  bool done = false;
  if (fixed_step_size > 0.0f) step_size = fixed_step_size;

  for (int st = 0; st < total_steps; ++st) {
    if (U && st >= noise_cols) return true;
    float u0 = U ? U[st] : 0.5f;
    float cdf = __fmul_rn(__fadd_rn((float)st, u0), step_size);
    while (cdf > cdf_hi) {
      if (!emit(I[bin], __fmul_rn(__fadd_rn(cmax, z_low), 0.5f), __fsub_rn(cmax, z_low)))
        return true;
      bin++;
      if (bin >= H || I[bin] == -1) { done = true; break; }
      cmin = lo[bin]; cmax = hi[bin];
      cdf_lo = cdf_hi;
      cdf_hi = __fadd_rn(cdf_hi, pr[bin]);
      z_low = cmin;
    }
    if (done) break;
    float u = __fdiv_rn(__fsub_rn(cdf, cdf_lo), __fsub_rn(cdf_hi, cdf_lo));
    float z = __fmaf_rn(u, __fsub_rn(cmax, cmin), cmin);
    if (!emit(I[bin], __fmul_rn(__fadd_rn(z, z_low), 0.5f), __fsub_rn(z, z_low))) return true;
    z_low = z;
  }
  // Tail: the reference runs it even after `done` (`~done` is always true),
  // re-emitting the last partial segment; with bin == H it reads the first
  // id of the next row in memory, and it tests emptiness on the block's
  // first row (fairnr/clib/src/sample_gpu.cu:188-201).
  while (z_low < cmax) {
    int32_t id;
    if (bin < H) id = I[bin];
    else id = (nxt >= 0) ? pts_all[nxt * H] : -1;
    if (!emit(id, __fmul_rn(__fadd_rn(cmax, z_low), 0.5f), __fsub_rn(cmax, z_low))) return true;
    bin++;
    if (bin >= H || I0[bin] == -1) break;
    cmin = lo[bin]; cmax = hi[bin];
    z_low = cmin;
  }
  return false;
}

// Rows the reference's tail reads outside a ray's own row, from the launch
// layout (see include/nsvf_gb300.h): tail row and next row of ray r.
__device__ __forceinline__ void icdf_rows(int64_t r, int64_t K, int64_t C, int64_t N, int64_t G,
                                          int64_t &tail, int64_t &nxt) {
  int64_t g = r / K, i = r % K;
  int64_t c0 = (i / C) * C, W = min(C, K - c0), ii = i - c0;
  tail = g * K + c0;
  if (tail >= N) tail = 0;
  if (ii + 1 < W) nxt = r + 1;
  else nxt = (g + 1 < G) ? (g + 1) * K + c0 : -1;
  if (nxt >= N) nxt = 0;
}

struct RowEmit {
  int32_t *SI;
  float *SD, *SS;
  int M, s, valid;
  __device__ bool operator()(int32_t id, float depth, float dist) {
    if (s >= M) return false;
    SI[s] = id; SD[s] = depth; SS[s] = dist;
    valid += (id != -1);
    ++s;
    return true;
  }
};

// One thread per ray: the padded [rows, M] outputs of the reference op.
__global__ void __launch_bounds__(kBlock) inverse_cdf_kernel(
    int64_t rows, int H, int M, int noise_stride, float fixed_step_size,
    const int32_t *__restrict__ pts_idx, const float *__restrict__ min_depth,
    const float *__restrict__ max_depth, const float *__restrict__ noise,
    const float *__restrict__ probs, const float *__restrict__ steps, int64_t K, int64_t C,
    int64_t N, int64_t G, int32_t *__restrict__ s_idx, float *__restrict__ s_depth,
    float *__restrict__ s_dist, int32_t *__restrict__ max_len, int32_t *__restrict__ err) {
  int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  bool live = r < rows;
  int valid = 0;
  if (live) {
    int64_t tail, nxt;
    icdf_rows(r, K, C, N, G, tail, nxt);
    RowEmit em{s_idx + r * M, s_depth + r * M, s_dist + r * M, M, 0, 0};
    bool overflow = icdf_walk(H, pts_idx + r * H, pts_idx + tail * H, pts_idx, nxt,
                              min_depth + r * H, max_depth + r * H, probs + r * H, steps[r],
                              noise ? noise + r * noise_stride : nullptr, noise_stride,
                              fixed_step_size, em);
    for (int q = em.s; q < M; ++q) { em.SI[q] = -1; em.SD[q] = 0.0f; em.SS[q] = 0.0f; }
    valid = em.valid;
    if (overflow && err) atomicOr(err, 2);
  }
  warp_max_atomic(max_len, valid, live);
}

// Served path, pass 1: number of valid (id != -1) samples of each ray.
struct CountEmit {
  int n;
  __device__ bool operator()(int32_t id, float, float) {
    n += (id != -1);
    return true;
  }
};

// With n_dev the number of rows (hit rays) is read on the device and the
// launch layout is the reference wrapper's for that many rays (200 blocks,
// 800-column launches); rows past it get count 0.
__device__ __forceinline__ bool dyn_rows(const int64_t *n_dev, int64_t cap, int64_t &rows,
                                         int64_t &K, int64_t &C, int64_t &N, int64_t &G) {
  if (!n_dev) return false;
  int64_t n = *n_dev;
  rows = n < 0 ? 0 : (n < cap ? n : cap);
  N = rows;
  G = 200;
  K = (N + G - 1) / G;
  if (K < 1) K = 1;
  C = 800;
  return true;
}

// With a piece table, the hit rows are the concatenation of independent
// pieces (pixel ranges of different frames packed into one serving chunk):
// piece p owns rows [piece_rows[p], piece_rows[p + 1]) (max_pieces + 1
// ascending entries; rows past the last entry belong to the last piece), and
// each piece gets the reference wrapper's layout for its own row count, as if
// it had been launched alone. A piece's results then do not depend on what
// else shares the chunk.
__device__ __forceinline__ void piece_rows_of(int64_t r, const int64_t *__restrict__ piece_rows,
                                              int max_pieces, int64_t &tail, int64_t &nxt) {
  int lo = 0, hi = max_pieces;   // piece_rows[lo] <= r; find the last such lo < max_pieces
  while (hi - lo > 1) {
    const int mid = (lo + hi) >> 1;
    if (piece_rows[mid] <= r) lo = mid;
    else hi = mid;
  }
  const int64_t base = piece_rows[lo];
  int64_t end = piece_rows[lo + 1];
  if (end <= r) end = r + 1;
  const int64_t N = end - base, G = 200;
  int64_t K = (N + G - 1) / G;
  if (K < 1) K = 1;
  icdf_rows(r - base, K, 800, N, G, tail, nxt);
  tail += base;
  if (nxt >= 0) nxt += base;
}

__device__ __forceinline__ void row_layout(int64_t r, int64_t K, int64_t C, int64_t N, int64_t G,
                                           const int64_t *__restrict__ piece_rows, int max_pieces,
                                           int64_t &tail, int64_t &nxt) {
  if (piece_rows) piece_rows_of(r, piece_rows, max_pieces, tail, nxt);
  else icdf_rows(r, K, C, N, G, tail, nxt);
}

__global__ void __launch_bounds__(kBlock) icdf_count_kernel(
    int64_t rows, int H, const int32_t *__restrict__ pts_idx, const float *__restrict__ min_depth,
    const float *__restrict__ max_depth, const float *__restrict__ probs,
    const float *__restrict__ steps, int64_t K, int64_t C, int64_t N, int64_t G,
    const int64_t *__restrict__ n_dev, int32_t *__restrict__ count,
    const int64_t *__restrict__ piece_rows, int max_pieces) {
  int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  int64_t cap = rows;
  dyn_rows(n_dev, cap, rows, K, C, N, G);
  if (r >= cap) return;
  if (r >= rows) { count[r] = 0; return; }
  int64_t tail, nxt;
  row_layout(r, K, C, N, G, piece_rows, max_pieces, tail, nxt);
  CountEmit em{0};
  icdf_walk(H, pts_idx + r * H, pts_idx + tail * H, pts_idx, nxt, min_depth + r * H,
            max_depth + r * H, probs + r * H, steps[r], nullptr, 0, -1.0f, em);
  count[r] = em.n;
}

// Served path, pass 2: the valid samples of every ray, compacted in ray
// order at offset[r]: voxel id, (x, y, z, clamped distance) and depth,
// with x = o + d * t as the renderer computes it.
struct CompactEmit {
  int32_t *vox;
  float4 *xyzd;
  float *depth;
  float ox, oy, oz, dx, dy, dz;
  int64_t pos, end;
  __device__ bool operator()(int32_t id, float t, float dist) {
    if (id == -1) return true;
    if (pos >= end) return false;
    vox[pos] = id;
    xyzd[pos] = make_float4(__fadd_rn(ox, __fmul_rn(dx, t)), __fadd_rn(oy, __fmul_rn(dy, t)),
                            __fadd_rn(oz, __fmul_rn(dz, t)), fmaxf(dist, 0.0f));
    depth[pos] = t;
    ++pos;
    return true;
  }
};

__global__ void __launch_bounds__(kBlock) icdf_compact_kernel(
    int64_t rows, int H, const int32_t *__restrict__ pts_idx, const float *__restrict__ min_depth,
    const float *__restrict__ max_depth, const float *__restrict__ probs,
    const float *__restrict__ steps, int64_t K, int64_t C, int64_t N, int64_t G,
    const int64_t *__restrict__ n_dev, const float *__restrict__ ray_start,
    int64_t ray_start_stride, const float *__restrict__ ray_dir,
    const int64_t *__restrict__ ray_index, const int64_t *__restrict__ offset,
    int64_t sample_cap, int32_t *__restrict__ vox, float4 *__restrict__ xyzd,
    float *__restrict__ depth, int32_t *__restrict__ err, const int64_t *__restrict__ piece_rows,
    int max_pieces) {
  int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  int64_t cap = rows;
  dyn_rows(n_dev, cap, rows, K, C, N, G);
  if (r >= rows) return;
  int64_t tail, nxt;
  row_layout(r, K, C, N, G, piece_rows, max_pieces, tail, nxt);
  // the ray's origin/direction: row r of the ray arrays, or row ray_index[r]
  int64_t rr = ray_index ? ray_index[r] : r;
  const float *o = ray_start + rr * ray_start_stride;
  int64_t end = offset[r + 1];
  if (end > sample_cap) {
    if (err) atomicOr(err, 2);
    end = sample_cap;
  }
  CompactEmit em{vox, xyzd, depth, o[0], o[1], o[2], ray_dir[rr * 3], ray_dir[rr * 3 + 1],
                 ray_dir[rr * 3 + 2], offset[r] < end ? offset[r] : end, end};
  bool overflow = icdf_walk(H, pts_idx + r * H, pts_idx + tail * H, pts_idx, nxt,
                            min_depth + r * H, max_depth + r * H, probs + r * H, steps[r],
                            nullptr, 0, -1.0f, em);
  if ((overflow || em.pos != em.end) && err) atomicOr(err, 2);
}

// ------------------------------------------------------------------------
// Served path, warp per ray. The walk above emits, for a ray with B valid
// bins (ids before the first -1) and T = ceil(steps) jittered steps at
// cdf_t = (t + 0.5) * step, this sequence: for each bin b, the steps that
// land in it, then (when a later step passes the bin's upper CDF bound) the
// bin's closing segment; after the last valid bin is closed the walk is
// done; then the tail loop. With sf[b + 1] = #{t : cdf_t <= cdf_hi[b]} (a
// binary search, cdf_t is increasing) every position is closed-form:
//   step t in bin b          at t + b,
//   closing segment of bin b at sf[b + 1] + b,   emitted iff sf[b + 1] < T,
// and a step's z_low is the previous step's z when that step is in the same
// bin, else the bin's min depth. So 32 lanes place 32 consecutive samples
// at once, with the walk's exact FP32 operations, and write them coalesced.
// The CDF bounds are the walk's sequential FP32 prefix (one lane); the tail
// loop runs on one lane. Rows with max_hits > kMaxH use the per-thread walk.
constexpr int kMaxH = 128;
constexpr int kWarpRays = 8;                 // warps (rays in flight) per block

struct RayTab {
  float lo[kMaxH], hi[kMaxH], cdf_hi[kMaxH];
  int32_t id[kMaxH];
  int sf[kMaxH + 1];
  int end[kMaxH];
};

__device__ __forceinline__ float tab_cdf(int t, float step) {
  return __fmul_rn(__fadd_rn((float)t, 0.5f), step);
}

// z of step t in bin b (the walk's in-bin placement)
__device__ __forceinline__ float tab_z(const RayTab &T, int t, int b, float step) {
  float cl = b > 0 ? T.cdf_hi[b - 1] : 0.0f;
  float u = __fdiv_rn(__fsub_rn(tab_cdf(t, step), cl), __fsub_rn(T.cdf_hi[b], cl));
  return __fmaf_rn(u, __fsub_rn(T.hi[b], T.lo[b]), T.lo[b]);
}

// z_low of bin b's closing segment: its last step's z, or its min depth
__device__ __forceinline__ float tab_zlow_close(const RayTab &T, int b, float step) {
  return T.sf[b + 1] > T.sf[b] ? tab_z(T, T.sf[b + 1] - 1, b, step) : T.lo[b];
}

struct WarpRay {
  int B, nb, M, total;
  float step;
  bool done;
};

// Builds the ray's table (all 32 lanes; returns the same WarpRay on every
// lane). B == 0 (an empty first slot) is left to the caller.
__device__ __forceinline__ WarpRay build_tab(RayTab &T, int H, const int32_t *__restrict__ I,
                                             const float *__restrict__ lo,
                                             const float *__restrict__ hi,
                                             const float *__restrict__ pr, float steps, int lane) {
  for (int b = lane; b < H; b += 32) { T.id[b] = I[b]; T.lo[b] = lo[b]; T.hi[b] = hi[b]; }
  __syncwarp();
  WarpRay w;
  w.step = __double2float_rn(__ddiv_rn(1.0, (double)steps));
  w.total = (int)ceilf(steps);
  int B = H;
  for (int b0 = 0; b0 < H; b0 += 32) {
    uint32_t m = __ballot_sync(0xffffffffu, b0 + lane < H && T.id[b0 + lane] == -1);
    if (m) { B = b0 + __ffs(m) - 1; break; }
  }
  w.B = B;
  if (lane == 0) {
    float c = pr[0];
    if (B > 0) T.cdf_hi[0] = c;
    for (int b = 1; b < B; ++b) { c = __fadd_rn(c, pr[b]); T.cdf_hi[b] = c; }
    T.sf[0] = 0;
  }
  __syncwarp();
  for (int b = lane; b < B; b += 32) {
    const float bound = T.cdf_hi[b];
    int a = 0, e = w.total;
    while (a < e) {
      int mid = (a + e) >> 1;
      if (tab_cdf(mid, w.step) <= bound) a = mid + 1;
      else e = mid;
    }
    T.sf[b + 1] = a;
  }
  __syncwarp();
  int nb = 0;
  for (int b0 = 0; b0 < B; b0 += 32)
    nb += __popc(__ballot_sync(0xffffffffu, b0 + lane < B && T.sf[b0 + lane + 1] < w.total));
  for (int b = lane; b < nb; b += 32) T.end[b] = T.sf[b + 1] + b + 1;
  __syncwarp();
  w.nb = nb;
  w.done = B > 0 && T.sf[B] < w.total;
  w.M = B > 0 ? T.sf[B] + nb : 0;
  return w;
}

// Main-sequence sample j (0 <= j < M): voxel id, depth, distance, in two
// steps so that a warp can pass each step's depth to the next sample's lane.
// tab_step finds sample j's bin b and, for a step sample (not b's closing
// segment), its step st and depth z. tab_finish takes z_prev, the depth of
// sample j - 1, which is the lower edge whenever sample j - 1 is a step of
// the same bin (st > sf[b] for a step; sf[b + 1] > sf[b] for the closing
// segment), and gives the sample's id, depth t and distance.
struct TabStep {
  int b = 0, st = 0;
  bool closing = false;
  float z = 0.0f;
};

__device__ __forceinline__ TabStep tab_step(const RayTab &T, const WarpRay &w, int j) {
  TabStep sp;
  int a = 0, e = w.nb;
  while (a < e) {
    int mid = (a + e) >> 1;
    if (T.end[mid] <= j) a = mid + 1;
    else e = mid;
  }
  sp.b = a;
  sp.closing = a < w.nb && j == T.end[a] - 1;
  if (!sp.closing) {
    sp.st = j - a;
    sp.z = tab_z(T, sp.st, a, w.step);
  }
  return sp;
}

__device__ __forceinline__ void tab_finish(const RayTab &T, const WarpRay &w, const TabStep &sp,
                                           float z_prev, int32_t &id, float &t, float &dist) {
  const int b = sp.b;
  id = T.id[b];
  if (sp.closing) {
    // tab_zlow_close: bin b's last step (sample j - 1), or its min depth
    float zl = T.sf[b + 1] > T.sf[b] ? z_prev : T.lo[b];
    t = __fmul_rn(__fadd_rn(T.hi[b], zl), 0.5f);
    dist = __fsub_rn(T.hi[b], zl);
  } else {
    // the previous step of this bin is sample j - 1
    float zl = sp.st > T.sf[b] ? z_prev : T.lo[b];
    t = __fmul_rn(__fadd_rn(sp.z, zl), 0.5f);
    dist = __fsub_rn(sp.z, zl);
  }
}

// The tail loop of the walk from its end state, calling emit(id, t, dist).
template <typename Emit>
__device__ __forceinline__ void tab_tail(const RayTab &T, const WarpRay &w, int H,
                                         const int32_t *__restrict__ I0,
                                         const int32_t *__restrict__ pts_all, int64_t nxt,
                                         Emit &emit) {
  int bin;
  float cmax, z_low;
  if (w.done) {
    bin = w.B; cmax = T.hi[w.B - 1]; z_low = tab_zlow_close(T, w.B - 1, w.step);
  } else if (w.total > 0) {
    bin = w.nb; cmax = T.hi[w.nb]; z_low = tab_z(T, w.total - 1, w.nb, w.step);
  } else {
    bin = 0; cmax = T.hi[0]; z_low = T.lo[0];
  }
  while (z_low < cmax) {
    int32_t id;
    if (bin < H) id = T.id[bin];
    else id = (nxt >= 0) ? pts_all[nxt * H] : -1;
    emit(id, __fmul_rn(__fadd_rn(cmax, z_low), 0.5f), __fsub_rn(cmax, z_low));
    bin++;
    if (bin >= H || I0[bin] == -1) break;
    cmax = T.hi[bin];
    z_low = T.lo[bin];
  }
}

struct TailCount {
  int n;
  __device__ void operator()(int32_t id, float, float) { n += (id != -1); }
};

struct TailWrite {
  int32_t *vox;
  float4 *xyzd;
  float *depth;
  float ox, oy, oz, dx, dy, dz;
  int64_t pos, end;
  bool over;
  __device__ void operator()(int32_t id, float t, float dist) {
    if (id == -1) return;
    if (pos >= end) { over = true; return; }
    vox[pos] = id;
    xyzd[pos] = make_float4(__fadd_rn(ox, __fmul_rn(dx, t)), __fadd_rn(oy, __fmul_rn(dy, t)),
                            __fadd_rn(oz, __fmul_rn(dz, t)), fmaxf(dist, 0.0f));
    depth[pos] = t;
    ++pos;
  }
};

// The samples of row r (table T, walk state w, built by build_tab) written
// to [start, end) of the compacted buffers, clipped to sample_cap; a count
// that differs from end - start, or an end past sample_cap, sets bit 2 of
// *err. All 32 lanes call it.
__device__ __forceinline__ void warp_write_samples(
    const RayTab &T, const WarpRay &w, int H, int64_t r, int64_t tail, int64_t nxt, int lane,
    const int32_t *__restrict__ pts_idx, const float *__restrict__ min_depth,
    const float *__restrict__ max_depth, const float *__restrict__ probs,
    const float *__restrict__ steps, const float *__restrict__ ray_start,
    int64_t ray_start_stride, const float *__restrict__ ray_dir,
    const int64_t *__restrict__ ray_index, int64_t start, int64_t end, int64_t sample_cap,
    int32_t *__restrict__ vox, float4 *__restrict__ xyzd, float *__restrict__ depth,
    int32_t *__restrict__ err) {
  const int32_t *I = pts_idx + r * H;
  const int64_t rr = ray_index ? ray_index[r] : r;
  const float *o = ray_start + rr * ray_start_stride;
  if (w.B == 0) {
    // an empty first slot: the per-thread walk on lane 0
    if (lane == 0) {
      int64_t e = end < sample_cap ? end : sample_cap;
      CompactEmit em{vox, xyzd, depth, o[0], o[1], o[2], ray_dir[rr * 3], ray_dir[rr * 3 + 1],
                     ray_dir[rr * 3 + 2], start < e ? start : e, e};
      bool over = icdf_walk(H, I, pts_idx + tail * H, pts_idx, nxt, min_depth + r * H,
                            max_depth + r * H, probs + r * H, steps[r], nullptr, 0, -1.0f, em);
      if ((over || em.pos != end) && err) atomicOr(err, 2);
    }
    return;
  }
  const float ox = o[0], oy = o[1], oz = o[2];
  const float dx = ray_dir[rr * 3], dy = ray_dir[rr * 3 + 1], dz = ray_dir[rr * 3 + 2];
  const int64_t base = start, lim = end < sample_cap ? end : sample_cap;
  // Sample j's lower edge is sample j - 1's depth z when both are steps of
  // one bin: lane - 1 computed it (lane 31 of the previous round for lane
  // 0), so each step's division runs once.
  float z_last = 0.0f;
  for (int j0 = 0; j0 < w.M; j0 += 32) {
    const int j = j0 + lane;
    TabStep sp;
    if (j < w.M) sp = tab_step(T, w, j);
    float z_prev = __shfl_up_sync(0xffffffffu, sp.z, 1);
    if (lane == 0) z_prev = z_last;
    z_last = __shfl_sync(0xffffffffu, sp.z, 31);
    if (j < w.M) {
      int32_t id;
      float t, dist;
      tab_finish(T, w, sp, z_prev, id, t, dist);
      const int64_t pos = base + j;
      if (pos < lim) {
        vox[pos] = id;
        xyzd[pos] = make_float4(__fadd_rn(ox, __fmul_rn(dx, t)), __fadd_rn(oy, __fmul_rn(dy, t)),
                                __fadd_rn(oz, __fmul_rn(dz, t)), fmaxf(dist, 0.0f));
        depth[pos] = t;
      }
    }
  }
  if (lane == 0) {
    TailWrite tw{vox, xyzd, depth, ox, oy, oz, dx, dy, dz, base + w.M, lim, false};
    if (base + w.M > lim) tw.over = true;
    tab_tail(T, w, H, pts_idx + tail * H, pts_idx, nxt, tw);
    if ((tw.over || tw.pos != end || end > sample_cap) && err) atomicOr(err, 2);
  }
}

// The number of samples of row r (lane 0's value; the table is built).
__device__ __forceinline__ int warp_count_samples(const RayTab &T, const WarpRay &w, int H,
                                                  int64_t r, int64_t tail, int64_t nxt, int lane,
                                                  const int32_t *__restrict__ pts_idx,
                                                  const float *__restrict__ min_depth,
                                                  const float *__restrict__ max_depth,
                                                  const float *__restrict__ probs,
                                                  const float *__restrict__ steps) {
  int n = 0;
  if (lane == 0) {
    if (w.B == 0) {
      CountEmit em{0};
      icdf_walk(H, pts_idx + r * H, pts_idx + tail * H, pts_idx, nxt, min_depth + r * H,
                max_depth + r * H, probs + r * H, steps[r], nullptr, 0, -1.0f, em);
      n = em.n;
    } else {
      TailCount tc{0};
      tab_tail(T, w, H, pts_idx + tail * H, pts_idx, nxt, tc);
      n = w.M + tc.n;
    }
  }
  return n;
}

// WRITE = false: count[r] = number of valid samples of row r (rows past the
// device-side row count get 0). WRITE = true: the samples, compacted at
// offset[r].
template <bool WRITE>
__global__ void __launch_bounds__(32 * kWarpRays) icdf_warp_kernel(
    int64_t rows, int H, const int32_t *__restrict__ pts_idx, const float *__restrict__ min_depth,
    const float *__restrict__ max_depth, const float *__restrict__ probs,
    const float *__restrict__ steps, int64_t K, int64_t C, int64_t N, int64_t G,
    const int64_t *__restrict__ n_dev, int32_t *__restrict__ count,
    const float *__restrict__ ray_start, int64_t ray_start_stride,
    const float *__restrict__ ray_dir, const int64_t *__restrict__ ray_index,
    const int64_t *__restrict__ offset, int64_t sample_cap, int32_t *__restrict__ vox,
    float4 *__restrict__ xyzd, float *__restrict__ depth, int32_t *__restrict__ err,
    const int64_t *__restrict__ piece_rows, int max_pieces) {
  __shared__ RayTab tabs[kWarpRays];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  RayTab &T = tabs[wib];
  const int64_t cap = rows;
  dyn_rows(n_dev, cap, rows, K, C, N, G);
  const int64_t stride = (int64_t)gridDim.x * kWarpRays;
  for (int64_t r = (int64_t)blockIdx.x * kWarpRays + wib; r < cap; r += stride) {
    if (r >= rows) {
      if (!WRITE && lane == 0) count[r] = 0;
      continue;
    }
    int64_t tail, nxt;
    row_layout(r, K, C, N, G, piece_rows, max_pieces, tail, nxt);
    const int32_t *I = pts_idx + r * H;
    WarpRay w = build_tab(T, H, I, min_depth + r * H, max_depth + r * H, probs + r * H,
                          steps[r], lane);
    if (!WRITE) {
      const int n = warp_count_samples(T, w, H, r, tail, nxt, lane, pts_idx, min_depth,
                                       max_depth, probs, steps);
      if (lane == 0) count[r] = n;
    } else {
      warp_write_samples(T, w, H, r, tail, nxt, lane, pts_idx, min_depth, max_depth, probs, steps,
                         ray_start, ray_start_stride, ray_dir, ray_index, offset[r],
                         offset[r + 1], sample_cap, vox, xyzd, depth, err);
    }
    __syncwarp();                          // the table is rebuilt for the next ray
  }
}

int scan_sms() {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
  }
  return sms;
}

// Blocks for the warp-per-ray kernels: enough warps to cover the rows (or
// the capacity), at most 16 blocks of 8 warps per SM (grid-stride beyond).
int warp_grid(int64_t rows) {
  static int sms = 0;
  if (!sms) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms < 1) sms = 1;
  }
  int64_t want = (rows + kWarpRays - 1) / kWarpRays;
  int64_t lim = (int64_t)sms * 16;
  return (int)(want < 1 ? 1 : (want < lim ? want : lim));
}

// Count and compaction in one pass (served path, warp per ray). Blocks take
// chunks of kScanWarps consecutive rows in ticket order (scan[0]); a block
// counts its rows' samples, publishes the chunk's count in scan[1 + c]
// (kScanAgg), finds the samples of all earlier chunks by a look-back over
// their published words (one warp, 32 chunks per step, stopping at the
// nearest chunk whose inclusive total is known: kScanInc), publishes its own
// inclusive total, and writes its rows' samples from there. offset[r] is the
// exclusive prefix sum of the counts, as the count pass and a prefix sum
// give it; the total is written to offset[rows] and offset[rows_cap]. A
// chunk's predecessors took their tickets first and publish their counts
// before they look back, so every wait ends; each is still bounded (bit 8
// of *err when one gives up).
constexpr int kScanWarps = 4;      // rays per block (4: 0.332 ms, 8: 0.338, 16: 0.359 on the c2 frame)
constexpr unsigned long long kScanAgg = 1ull << 62, kScanInc = 2ull << 62;
constexpr unsigned long long kScanVal = (1ull << 62) - 1;

__device__ __forceinline__ unsigned long long scan_load(const unsigned long long *p) {
  return *reinterpret_cast<const volatile unsigned long long *>(p);
}

__global__ void __launch_bounds__(32 * kScanWarps) icdf_scan_kernel(
    int64_t rows_cap, int H, const int32_t *__restrict__ pts_idx,
    const float *__restrict__ min_depth, const float *__restrict__ max_depth,
    const float *__restrict__ probs, const float *__restrict__ steps,
    const int64_t *__restrict__ n_dev, const float *__restrict__ ray_start,
    int64_t ray_start_stride, const float *__restrict__ ray_dir,
    const int64_t *__restrict__ ray_index, int64_t *__restrict__ offset, int64_t sample_cap,
    int32_t *__restrict__ vox, float4 *__restrict__ xyzd, float *__restrict__ depth,
    unsigned long long *__restrict__ scan, int32_t *__restrict__ err,
    const int64_t *__restrict__ piece_rows, int max_pieces) {
  __shared__ RayTab tabs[kScanWarps];
  __shared__ int s_cnt[kScanWarps];
  __shared__ long long s_chunk, s_base;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  RayTab &T = tabs[wib];
  int64_t rows = rows_cap, K = 1, C = 1, N = 1, G = 1;
  dyn_rows(n_dev, rows_cap, rows, K, C, N, G);
  const int64_t n_chunks = (rows + kScanWarps - 1) / kScanWarps;
  if (n_chunks == 0) {
    if (blockIdx.x == 0 && threadIdx.x == 0) offset[0] = offset[rows_cap] = 0;
    return;
  }
  unsigned long long *status = scan + 1;
  for (;;) {
    if (threadIdx.x == 0) s_chunk = (long long)atomicAdd(scan, 1ull);
    __syncthreads();
    const int64_t c = s_chunk;
    if (c >= n_chunks) break;
    const int64_t r = c * kScanWarps + wib;
    WarpRay w{};
    int64_t tail = 0, nxt = -1;
    int n = 0;
    if (r < rows) {
      row_layout(r, K, C, N, G, piece_rows, max_pieces, tail, nxt);
      w = build_tab(T, H, pts_idx + r * H, min_depth + r * H, max_depth + r * H, probs + r * H,
                    steps[r], lane);
      n = warp_count_samples(T, w, H, r, tail, nxt, lane, pts_idx, min_depth, max_depth, probs,
                             steps);
    }
    if (lane == 0) s_cnt[wib] = n;
    __syncthreads();
    if (wib == 0) {
      unsigned long long agg = 0;
      for (int k = 0; k < kScanWarps; ++k) agg += (unsigned long long)s_cnt[k];
      unsigned long long prefix = 0;
      if (c == 0) {
        if (lane == 0) atomicExch(status, kScanInc | agg);
      } else {
        if (lane == 0) atomicExch(status + c, kScanAgg | agg);
        // look back 32 chunks at a time: lane k reads chunk j - k
        int64_t j = c - 1;
        bool ok = true;
        for (;;) {
          const int64_t jj = j - lane;
          unsigned long long v = jj >= 0 ? scan_load(status + jj) : kScanInc;
          for (int it = 0; !__all_sync(0xffffffffu, v != 0ull); ++it) {
            if (it > (1 << 22)) { ok = false; break; }
            __nanosleep(32);
            if (v == 0ull) v = scan_load(status + jj);
          }
          if (!ok) break;
          // the nearest chunk with an inclusive total ends this step's sum
          const unsigned inc = __ballot_sync(0xffffffffu, (v & kScanInc) != 0ull);
          const int stop = inc ? __ffs(inc) - 1 : 31;
          unsigned long long part = lane <= stop ? (v & kScanVal) : 0ull;
          for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
          prefix += part;
          if (inc) break;
          j -= 32;
        }
        if (!ok && lane == 0 && err) atomicOr(err, 8);
        if (lane == 0) atomicExch(status + c, kScanInc | (prefix + agg));
      }
      if (lane == 0) {
        s_base = (long long)prefix;
        if (c == n_chunks - 1) offset[rows] = offset[rows_cap] = (int64_t)(prefix + agg);
      }
    }
    __syncthreads();
    if (r < rows) {
      int64_t start = s_base;
      for (int k = 0; k < wib; ++k) start += s_cnt[k];
      if (lane == 0) offset[r] = start;
      warp_write_samples(T, w, H, r, tail, nxt, lane, pts_idx, min_depth, max_depth, probs, steps,
                         ray_start, ray_start_stride, ray_dir, ray_index, start, start + s_cnt[wib],
                         sample_cap, vox, xyzd, depth, err);
    }
    __syncthreads();                      // tables and s_cnt are reused by the next chunk
  }
}

// Uniform sampler (fairnr/clib/src/sample_gpu.cu:15-106): merge interval
// starts, interval ends and jittered steps into one sorted depth list in the
// output row, then turn it into midpoints/lengths and keep those inside a
// voxel, compacting in place.
__global__ void __launch_bounds__(kBlock) uniform_kernel(
    int64_t rows, int H, int M, float step_size, const int32_t *__restrict__ pts_idx,
    const float *__restrict__ min_depth, const float *__restrict__ max_depth,
    const float *__restrict__ noise, int32_t *__restrict__ s_idx, float *__restrict__ s_depth,
    float *__restrict__ s_dist, int32_t *__restrict__ err) {
  int64_t r = blockIdx.x * (int64_t)kBlock + threadIdx.x;
  if (r >= rows) return;
  const int32_t *I = pts_idx + r * H;
  const float *lo = min_depth + r * H, *hi = max_depth + r * H;
  const float *U = noise + r * M;
  int32_t *SI = s_idx + r * M;
  float *SD = s_depth + r * M, *SS = s_dist + r * M;
  for (int q = 0; q < M; ++q) { SI[q] = -1; SD[q] = 0.0f; SS[q] = 0.0f; }

  int s = 0, ucur = 0, umin = 0, umax = 0;
  float lmin, lmax, cur = 0.0f;
  bool overflow = false;
  while (true) {
    if (umax == H || ucur == M || I[umax] == -1) break;
    if (s >= M) { overflow = true; break; }
    lmin = (umin < H) ? lo[umin] : 10000.0f;
    lmax = (umax < H) ? hi[umax] : 10000.0f;
    cur = __fmaf_rn(__fadd_rn((float)ucur, U[ucur]), step_size, lo[0]);
    if (lmax <= cur && lmax <= lmin) {
      SD[s] = lmax; SI[s] = I[umax]; umax++; s++; continue;
    }
    if (cur <= lmin && cur <= lmax) {
      // umin == 0 only for a jitter of exactly 0: the reference then reads the
      // element before the row (the previous ray's last id).
      int64_t off = r * H + umin - 1;
      SD[s] = cur; SI[s] = (off >= 0) ? pts_idx[off] : -1; ucur++; s++; continue;
    }
    if (lmin <= cur && lmin <= lmax) {
      SD[s] = lmin; SI[s] = I[umin]; umin++; s++; continue;
    }
    break;  // NaN input: the reference would spin here forever
  }

  int step = 0;
  umin = 0; umax = 0;
  for (ucur = 0; ucur < M - 1; ucur++) {
    if (SI[ucur + 1] == -1) break;
    float l = SD[ucur], rr = SD[ucur + 1];
    SD[ucur] = __fmul_rn(__fadd_rn(l, rr), 0.5f);
    SS[ucur] = __fsub_rn(rr, l);
    if (umin < H && SD[ucur] >= lo[umin] && I[umin] > -1) umin++;
    if (umax < H && SD[ucur] >= hi[umax] && I[umax] > -1) umax++;
    if (umax == H || I[umax] == -1) break;
    if (umin - 1 == umax && SS[ucur] > 0) {
      SD[step] = SD[ucur]; SS[step] = SS[ucur]; SI[step] = SI[ucur]; step++;
    }
  }
  for (int q = step; q < M; ++q) SI[q] = -1;
  if (overflow && err) atomicOr(err, 2);
}

// Parallel uniform sampler: the pure-torch backup sampler of the reference's
// op set (fairnr/clib/__init__.py:303-349, `_parallel_ray_sampling`), here a
// warp per ray with its lists in shared memory. Per ray, with the H sorted
// hit slots (pts_idx, min m_i, max M_i; misses carry MAX_DEPTH):
//   u_k = m_0 + (k + j_k) * march for k < K (j_k = 0.5, or the clamped
//       jitter), taking the id of slot #{i : m_i <= u_k} - 1;
//   the 2H + K depths {M_i} u {m_i} u {u_k}, each with its id, sorted with
//       ties in that concatenation order (a stable sort): at a face shared
//       by two voxels the exit comes first, so the segment after it takes
//       the id of the voxel being entered (the reference's torch.sort leaves
//       that order unspecified; on the CPU it orders such ties both ways);
//   segment s between consecutive depths d_s, d_s+1: midpoint .5 (d_s +
//       d_s+1), length d_s+1 - d_s, the id of d_s; kept when #{i : m_i <=
//       mid} - 1 == #{i : M_i <= mid}, mid <= max_i M_i (MAX_DEPTH read as
//       0) and the length is not 0.
// The kept segments are written in order (count[r] of them), then -1 /
// MAX_DEPTH / 0 up to out_w. The sort is done as ranks: each boundary's rank
// among the 2H boundaries counts smaller values and equal values earlier in
// the concatenation; a boundary's merged position adds the steps strictly
// below it, a step's adds the boundaries at or below it (both lists are
// sorted, so binary searches). Shared memory per warp: 4 * (8H + 2N) bytes,
// N = 2H + K (raw boundaries and ids, sorted boundaries and ids, the merged
// depths and ids).
constexpr int kParWarps = 4;

__device__ __forceinline__ float par_step(int k, const float *__restrict__ J, float m0,
                                          float march) {
  const float j = J ? J[k] : 0.5f;
  return __fadd_rn(m0, __fmul_rn(__fadd_rn((float)k, j), march));
}

__global__ void __launch_bounds__(32 * kParWarps) parallel_sampling_kernel(
    int64_t rows, int H, int K, float march, const int32_t *__restrict__ pts_idx,
    const float *__restrict__ min_depth, const float *__restrict__ max_depth,
    const float *__restrict__ noise, int out_w, int32_t *__restrict__ s_idx,
    float *__restrict__ s_depth, float *__restrict__ s_dist, int32_t *__restrict__ count) {
  extern __shared__ float par_smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int N = 2 * H + K;
  float *bv = par_smem + (size_t)w * (8 * H + 2 * N);
  int32_t *bi = reinterpret_cast<int32_t *>(bv + 2 * H);
  float *sv = bv + 4 * H;
  int32_t *si = reinterpret_cast<int32_t *>(bv + 6 * H);
  float *mval = bv + 8 * H;
  int32_t *midx = reinterpret_cast<int32_t *>(bv + 8 * H + N);
  const int64_t warps = (int64_t)gridDim.x * kParWarps;
  for (int64_t r = blockIdx.x * (int64_t)kParWarps + w; r < rows; r += warps) {
    const int32_t *I = pts_idx + r * H;
    const float *lo = min_depth + r * H, *hi = max_depth + r * H;
    const float *J = noise ? noise + r * K : nullptr;
    // bv = [exits M_0..M_H-1, entries m_0..m_H-1]
    const float *mins = bv + H, *maxs = bv;
    float mx = 0.0f;
    for (int i = lane; i < H; i += 32) {
      const float a = lo[i], b = hi[i];
      bv[i] = b;
      bv[H + i] = a;
      bi[i] = bi[H + i] = I[i];
      const float bb = b == NSVF_MAX_DEPTH_F ? 0.0f : b;
      mx = fmaxf(mx, bb);
    }
    for (int o = 16; o > 0; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    __syncwarp();
    const float m0 = mins[0];
    // stable ranks of the 2H boundaries
    for (int e = lane; e < 2 * H; e += 32) {
      const float v = bv[e];
      int rank = 0;
      for (int f = 0; f < 2 * H; ++f) {
        const float u = bv[f];
        rank += (u < v || (u == v && f < e)) ? 1 : 0;
      }
      sv[rank] = v;
      si[rank] = bi[e];
    }
    __syncwarp();
    // the steps: merged position k + #{boundaries <= u}, id from the slot count
    for (int k = lane; k < K; k += 32) {
      const float u = par_step(k, J, m0, march);
      int a = 0, b = 2 * H;       // first boundary > u
      while (a < b) {
        const int m = (a + b) >> 1;
        if (sv[m] <= u) a = m + 1;
        else b = m;
      }
      int c = 0;
      for (int i = 0; i < H; ++i) c += (u >= mins[i]) ? 1 : 0;
      mval[k + a] = u;
      midx[k + a] = c >= 1 ? bi[H + c - 1] : -1;
    }
    // the boundaries: merged position q + #{steps < v}
    for (int q = lane; q < 2 * H; q += 32) {
      const float v = sv[q];
      int a = 0, b = K;           // first step >= v
      while (a < b) {
        const int m = (a + b) >> 1;
        if (par_step(m, J, m0, march) < v) a = m + 1;
        else b = m;
      }
      mval[q + a] = v;
      midx[q + a] = si[q];
    }
    __syncwarp();
    // segments, kept ones compacted in order
    int cnt = 0;
    for (int base = 0; base < N - 1; base += 32) {
      const int sgm = base + lane;
      bool keep = false;
      float mid = 0.0f, len = 0.0f;
      int32_t id = -1;
      if (sgm < N - 1) {
        const float a = mval[sgm], b = mval[sgm + 1];
        mid = __fmul_rn(0.5f, __fadd_rn(a, b));
        len = __fsub_rn(b, a);
        id = midx[sgm];
        int cmin = 0, cmax = 0;
        for (int i = 0; i < H; ++i) {
          cmin += (mid >= mins[i]) ? 1 : 0;
          cmax += (mid >= maxs[i]) ? 1 : 0;
        }
        keep = (cmin - 1 == cmax) && !(mid > mx) && !(len == 0.0f);
      }
      const unsigned m = __ballot_sync(0xffffffffu, keep);
      const int pos = cnt + __popc(m & ((1u << lane) - 1u));
      if (keep && pos < out_w) {
        s_idx[r * out_w + pos] = id;
        s_depth[r * out_w + pos] = mid;
        s_dist[r * out_w + pos] = len;
      }
      cnt += __popc(m);
    }
    for (int q = cnt + lane; q < out_w; q += 32) {
      s_idx[r * out_w + q] = -1;
      s_depth[r * out_w + q] = NSVF_MAX_DEPTH_F;
      s_dist[r * out_w + q] = 0.0f;
    }
    if (lane == 0 && count) count[r] = cnt;
    __syncwarp();
  }
}

}  // namespace

extern "C" {

int64_t nsvf_parallel_sampling_smem_bytes(int max_hits, int n_steps) {
  if (max_hits < 1 || n_steps < 0) return -1;
  const int64_t N = 2 * (int64_t)max_hits + n_steps;
  return 4 * (8 * (int64_t)max_hits + 2 * N);
}

int nsvf_parallel_ray_sampling(int64_t rows, int max_hits, int n_steps, float march_size,
                               const int32_t *pts_idx, const float *min_depth,
                               const float *max_depth, const float *noise, int out_width,
                               int32_t *sampled_idx, float *sampled_depth, float *sampled_dists,
                               int32_t *count, void *stream) {
  if (rows < 0 || max_hits < 1 || n_steps < 0 || out_width < 0) return NSVF_ERR_INVALID;
  if (rows == 0) return NSVF_OK;
  if (!pts_idx || !min_depth || !max_depth || (out_width > 0 && (!sampled_idx || !sampled_depth ||
      !sampled_dists)))
    return NSVF_ERR_INVALID;
  // all kParWarps warps' lists in one block's shared memory (<= 224 KB)
  const int64_t per_warp = nsvf_parallel_sampling_smem_bytes(max_hits, n_steps);
  const int64_t smem = per_warp * kParWarps;
  if (smem > 224 * 1024) return NSVF_ERR_CAPACITY;
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(parallel_sampling_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    return NSVF_ERR_CUDA;
  int64_t blocks = (rows + kParWarps - 1) / kParWarps;
  if (blocks > 152 * 16) blocks = 152 * 16;
  parallel_sampling_kernel<<<(int)blocks, 32 * kParWarps, (size_t)smem, (cudaStream_t)stream>>>(
      rows, max_hits, n_steps, march_size, pts_idx, min_depth, max_depth, noise, out_width,
      sampled_idx, sampled_depth, sampled_dists, count);
  return nsvf_launch_status();
}


int nsvf_inverse_cdf_sampling(int64_t rows, int max_hits, int max_steps, int noise_stride,
                              float fixed_step_size, const int32_t *pts_idx,
                              const float *min_depth, const float *max_depth, const float *noise,
                              const float *probs, const float *steps, const int64_t layout[4],
                              int32_t *sampled_idx, float *sampled_depth, float *sampled_dists,
                              int32_t *max_len, int32_t *err, void *stream) {
  if (rows < 0 || max_hits < 1 || max_steps < 1 || !layout || !pts_idx || !min_depth ||
      !max_depth || !probs || !steps || !sampled_idx || !sampled_depth || !sampled_dists)
    return NSVF_ERR_INVALID;
  if (noise && noise_stride < 1) return NSVF_ERR_INVALID;
  int64_t K = layout[0], C = layout[1], N = layout[2], G = layout[3];
  if (K < 1 || C < 1 || N < rows || G < 1 || G * K < N) return NSVF_ERR_INVALID;
  if (rows == 0) return NSVF_OK;
  inverse_cdf_kernel<<<nsvf_grid(rows, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
      rows, max_hits, max_steps, noise_stride, fixed_step_size, pts_idx, min_depth, max_depth,
      noise, probs, steps, K, C, N, G, sampled_idx, sampled_depth, sampled_dists, max_len, err);
  return nsvf_launch_status();
}

int nsvf_sample_count(int64_t rows, int max_hits, const int32_t *pts_idx, const float *min_depth,
                      const float *max_depth, const float *probs, const float *steps,
                      const int64_t layout[4], int32_t *count, void *stream) {
  if (rows < 0 || max_hits < 1 || !layout) return NSVF_ERR_INVALID;
  if (rows == 0) return NSVF_OK;
  if (!pts_idx || !min_depth || !max_depth || !probs || !steps || !count) return NSVF_ERR_INVALID;
  int64_t K = layout[0], C = layout[1], N = layout[2], G = layout[3];
  if (K < 1 || C < 1 || N < rows || G < 1 || G * K < N) return NSVF_ERR_INVALID;
  if (max_hits <= kMaxH)
    icdf_warp_kernel<false><<<warp_grid(rows), 32 * kWarpRays, 0, (cudaStream_t)stream>>>(
        rows, max_hits, pts_idx, min_depth, max_depth, probs, steps, K, C, N, G, nullptr, count,
        nullptr, 0, nullptr, nullptr, nullptr, 0, nullptr, nullptr, nullptr, nullptr, nullptr, 0);
  else
    icdf_count_kernel<<<nsvf_grid(rows, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
        rows, max_hits, pts_idx, min_depth, max_depth, probs, steps, K, C, N, G, nullptr, count,
        nullptr, 0);
  return nsvf_launch_status();
}

int nsvf_sample_compact(int64_t rows, int max_hits, const int32_t *pts_idx,
                        const float *min_depth, const float *max_depth, const float *probs,
                        const float *steps, const int64_t layout[4], const float *ray_start,
                        int64_t ray_start_stride, const float *ray_dir, const int64_t *offset,
                        int32_t *voxel, float *xyz_dist, float *depth, int32_t *err,
                        void *stream) {
  if (rows < 0 || max_hits < 1 || !layout || (ray_start_stride != 0 && ray_start_stride != 3))
    return NSVF_ERR_INVALID;
  if (rows == 0) return NSVF_OK;
  if (!pts_idx || !min_depth || !max_depth || !probs || !steps || !ray_start || !ray_dir ||
      !offset || !voxel || !xyz_dist || !depth || (((uintptr_t)xyz_dist) & 15))
    return NSVF_ERR_INVALID;
  int64_t K = layout[0], C = layout[1], N = layout[2], G = layout[3];
  if (K < 1 || C < 1 || N < rows || G < 1 || G * K < N) return NSVF_ERR_INVALID;
  if (max_hits <= kMaxH)
    icdf_warp_kernel<true><<<warp_grid(rows), 32 * kWarpRays, 0, (cudaStream_t)stream>>>(
        rows, max_hits, pts_idx, min_depth, max_depth, probs, steps, K, C, N, G, nullptr, nullptr,
        ray_start, ray_start_stride, ray_dir, nullptr, offset, INT64_MAX, voxel,
        (float4 *)xyz_dist, depth, err, nullptr, 0);
  else
    icdf_compact_kernel<<<nsvf_grid(rows, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
        rows, max_hits, pts_idx, min_depth, max_depth, probs, steps, K, C, N, G, nullptr, ray_start,
        ray_start_stride, ray_dir, nullptr, offset, INT64_MAX, voxel, (float4 *)xyz_dist, depth,
        err, nullptr, 0);
  return nsvf_launch_status();
}

int nsvf_sample_count_pieces(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                             const int32_t *pts_idx, const float *min_depth,
                             const float *max_depth, const float *probs, const float *steps,
                             const int64_t *piece_rows, int max_pieces, int32_t *count,
                             void *stream) {
  if (rows_cap < 0 || max_hits < 1 || !n_rows_dev || max_pieces < 0 ||
      (max_pieces > 0 && !piece_rows))
    return NSVF_ERR_INVALID;
  if (rows_cap == 0) return NSVF_OK;
  if (!pts_idx || !min_depth || !max_depth || !probs || !steps || !count) return NSVF_ERR_INVALID;
  const int64_t *pr = max_pieces > 0 ? piece_rows : nullptr;
  if (max_hits <= kMaxH)
    icdf_warp_kernel<false><<<warp_grid(rows_cap), 32 * kWarpRays, 0, (cudaStream_t)stream>>>(
        rows_cap, max_hits, pts_idx, min_depth, max_depth, probs, steps, 1, 1, 1, 1, n_rows_dev,
        count, nullptr, 0, nullptr, nullptr, nullptr, 0, nullptr, nullptr, nullptr, nullptr, pr,
        max_pieces);
  else
    icdf_count_kernel<<<nsvf_grid(rows_cap, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
        rows_cap, max_hits, pts_idx, min_depth, max_depth, probs, steps, 1, 1, 1, 1, n_rows_dev,
        count, pr, max_pieces);
  return nsvf_launch_status();
}

int nsvf_sample_count_dev(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                          const int32_t *pts_idx, const float *min_depth, const float *max_depth,
                          const float *probs, const float *steps, int32_t *count, void *stream) {
  return nsvf_sample_count_pieces(rows_cap, n_rows_dev, max_hits, pts_idx, min_depth, max_depth,
                                  probs, steps, nullptr, 0, count, stream);
}

int nsvf_sample_compact_pieces(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                               const int32_t *pts_idx, const float *min_depth,
                               const float *max_depth, const float *probs, const float *steps,
                               const int64_t *piece_rows, int max_pieces,
                               const float *ray_start, int64_t ray_start_stride,
                               const float *ray_dir, const int64_t *ray_index,
                               const int64_t *offset, int64_t sample_cap, int32_t *voxel,
                               float *xyz_dist, float *depth, int32_t *err, void *stream) {
  if (rows_cap < 0 || max_hits < 1 || !n_rows_dev || sample_cap < 0 ||
      (ray_start_stride != 0 && ray_start_stride != 3) || max_pieces < 0 ||
      (max_pieces > 0 && !piece_rows))
    return NSVF_ERR_INVALID;
  if (rows_cap == 0) return NSVF_OK;
  if (!pts_idx || !min_depth || !max_depth || !probs || !steps || !ray_start || !ray_dir ||
      !offset || !voxel || !xyz_dist || !depth || (((uintptr_t)xyz_dist) & 15))
    return NSVF_ERR_INVALID;
  const int64_t *pr = max_pieces > 0 ? piece_rows : nullptr;
  if (max_hits <= kMaxH)
    icdf_warp_kernel<true><<<warp_grid(rows_cap), 32 * kWarpRays, 0, (cudaStream_t)stream>>>(
        rows_cap, max_hits, pts_idx, min_depth, max_depth, probs, steps, 1, 1, 1, 1, n_rows_dev,
        nullptr, ray_start, ray_start_stride, ray_dir, ray_index, offset, sample_cap, voxel,
        (float4 *)xyz_dist, depth, err, pr, max_pieces);
  else
    icdf_compact_kernel<<<nsvf_grid(rows_cap, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
        rows_cap, max_hits, pts_idx, min_depth, max_depth, probs, steps, 1, 1, 1, 1, n_rows_dev,
        ray_start, ray_start_stride, ray_dir, ray_index, offset, sample_cap, voxel,
        (float4 *)xyz_dist, depth, err, pr, max_pieces);
  return nsvf_launch_status();
}

int nsvf_sample_compact_dev(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                            const int32_t *pts_idx, const float *min_depth,
                            const float *max_depth, const float *probs, const float *steps,
                            const float *ray_start, int64_t ray_start_stride,
                            const float *ray_dir, const int64_t *ray_index,
                            const int64_t *offset, int64_t sample_cap, int32_t *voxel,
                            float *xyz_dist, float *depth, int32_t *err, void *stream) {
  return nsvf_sample_compact_pieces(rows_cap, n_rows_dev, max_hits, pts_idx, min_depth,
                                    max_depth, probs, steps, nullptr, 0, ray_start,
                                    ray_start_stride, ray_dir, ray_index, offset, sample_cap,
                                    voxel, xyz_dist, depth, err, stream);
}

int64_t nsvf_sample_scan_bytes(int64_t rows_cap) {
  if (rows_cap < 0) return 0;
  return (int64_t)sizeof(unsigned long long) * (2 + (rows_cap + kScanWarps - 1) / kScanWarps);
}

int nsvf_sample_scan_compact_pieces(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                                    const int32_t *pts_idx, const float *min_depth,
                                    const float *max_depth, const float *probs,
                                    const float *steps, const int64_t *piece_rows, int max_pieces,
                                    const float *ray_start, int64_t ray_start_stride,
                                    const float *ray_dir, const int64_t *ray_index,
                                    int64_t *offset, int64_t sample_cap, int32_t *voxel,
                                    float *xyz_dist, float *depth, void *scan_ws,
                                    int64_t scan_ws_bytes, int32_t *err, void *stream) {
  if (rows_cap < 0 || max_hits < 1 || max_hits > kMaxH || !n_rows_dev || sample_cap < 0 ||
      (ray_start_stride != 0 && ray_start_stride != 3) || max_pieces < 0 ||
      (max_pieces > 0 && !piece_rows))
    return NSVF_ERR_INVALID;
  if (!offset) return NSVF_ERR_INVALID;
  if (rows_cap == 0) {
    return cudaMemsetAsync(offset, 0, sizeof(int64_t), (cudaStream_t)stream) == cudaSuccess
               ? NSVF_OK : NSVF_ERR_CUDA;
  }
  if (!pts_idx || !min_depth || !max_depth || !probs || !steps || !ray_start || !ray_dir ||
      !voxel || !xyz_dist || !depth || !scan_ws || (((uintptr_t)xyz_dist) & 15) ||
      (((uintptr_t)scan_ws) & 7))
    return NSVF_ERR_INVALID;
  const int64_t need = nsvf_sample_scan_bytes(rows_cap);
  if (scan_ws_bytes < need) return NSVF_ERR_CAPACITY;
  if (cudaMemsetAsync(scan_ws, 0, (size_t)need, (cudaStream_t)stream) != cudaSuccess)
    return NSVF_ERR_CUDA;
  const int64_t *pr = max_pieces > 0 ? piece_rows : nullptr;
  // 8 blocks of 4 warps per SM, taking chunks until none is left
  const int64_t want = (rows_cap + kScanWarps - 1) / kScanWarps, lim = 8 * (int64_t)scan_sms();
  icdf_scan_kernel<<<(int)(want < lim ? want : lim), 32 * kScanWarps, 0, (cudaStream_t)stream>>>(
      rows_cap, max_hits, pts_idx, min_depth, max_depth, probs, steps, n_rows_dev, ray_start,
      ray_start_stride, ray_dir, ray_index, offset, sample_cap, voxel, (float4 *)xyz_dist, depth,
      (unsigned long long *)scan_ws, err, pr, max_pieces);
  return nsvf_launch_status();
}

int nsvf_sample_scan_compact_dev(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                                 const int32_t *pts_idx, const float *min_depth,
                                 const float *max_depth, const float *probs, const float *steps,
                                 const float *ray_start, int64_t ray_start_stride,
                                 const float *ray_dir, const int64_t *ray_index, int64_t *offset,
                                 int64_t sample_cap, int32_t *voxel, float *xyz_dist, float *depth,
                                 void *scan_ws, int64_t scan_ws_bytes, int32_t *err,
                                 void *stream) {
  return nsvf_sample_scan_compact_pieces(rows_cap, n_rows_dev, max_hits, pts_idx, min_depth,
                                         max_depth, probs, steps, nullptr, 0, ray_start,
                                         ray_start_stride, ray_dir, ray_index, offset, sample_cap,
                                         voxel, xyz_dist, depth, scan_ws, scan_ws_bytes, err,
                                         stream);
}

int nsvf_uniform_ray_sampling(int b, int m, int max_hits, int max_steps, float step_size,
                              const int32_t *pts_idx, const float *min_depth,
                              const float *max_depth, const float *noise, int32_t *sampled_idx,
                              float *sampled_depth, float *sampled_dists, int32_t *err,
                              void *stream) {
  if (b < 0 || m < 0 || max_hits < 1 || max_steps < 1 || !pts_idx || !min_depth || !max_depth ||
      !noise || !sampled_idx || !sampled_depth || !sampled_dists)
    return NSVF_ERR_INVALID;
  int64_t rows = (int64_t)b * m;
  if (rows == 0) return NSVF_OK;
  uniform_kernel<<<nsvf_grid(rows, kBlock), kBlock, 0, (cudaStream_t)stream>>>(
      rows, max_hits, max_steps, step_size, pts_idx, min_depth, max_depth, noise, sampled_idx,
      sampled_depth, sampled_dists, err);
  return nsvf_launch_status();
}

}  // extern "C"
