/*
 * CPU oracle for the fairnr.clib ray/voxel ops.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker used by tests/, by
 * __graft_entry__.smoke() and by the cpu_baseline leg of bench.py. The
 * product path (nsvf_gb300) never links or calls it.
 *
 * Each function is a plain-C restatement of the reference's per-ray
 * algorithm, written for clarity, one ray at a time, with the reference's
 * memory layout ([b, m, ...] blocks) and its quirks kept:
 *
 *   or_slab             fairnr/clib/src/intersect_gpu.cu:73-122  (RayAABBIntersection)
 *   or_aabb_intersect   fairnr/clib/src/intersect_gpu.cu:125-167 + intersect.cpp:49-75
 *   or_svo_intersect    fairnr/clib/src/intersect_gpu.cu:170-237 + intersect.cpp:84-112
 *   or_ball_intersect   fairnr/clib/src/intersect_gpu.cu:15-70   + intersect.cpp:15-41
 *   or_triangle_intersect fairnr/clib/src/intersect_gpu.cu:238-337 + intersect.cpp:120-145
 *   or_uniform_sampling fairnr/clib/src/sample_gpu.cu:15-106     + sample.cpp:23-55
 *   or_inverse_cdf      fairnr/clib/src/sample_gpu.cu:108-202    + sample.cpp:58-96
 *   or_build_octree     fairnr/clib/src/octree.cpp:13-136
 *
 * Floating point. The reference is FP32 compiled by nvcc with default flags,
 * so `a + b * c` is contracted to one fused multiply-add. The oracle writes
 * those contractions as fmaf() (correctly rounded in C99) and everything else
 * as separate FP32 operations; build with -ffp-contract=off so the C compiler
 * adds no contraction of its own. The one deliberate difference: the
 * reference computes 1/dir with __fdividef (an approximate reciprocal whose
 * bits are not specified), the oracle with IEEE division. The CUDA product
 * uses the IEEE reciprocal too, so product and oracle agree bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define OR_MAX_DEPTH 10000.0f

/* Slab test of one ray against one axis-aligned cube (centre c, half size h).
 * Returns 1 and (t_low, t_high) on a hit, 0 on a miss. t_low is clipped at 0
 * and t_high starts at 1e5; comparisons with NaN are false, so a NaN axis is
 * skipped, exactly as in the reference. */
static int or_slab(const float o[3], const float d[3], const float c[3], float h,
                   float *t_lo, float *t_hi) {
  float lo = 0.0f, hi = 100000.0f;
  for (int a = 0; a < 3; ++a) {
    float inv = 1.0f / d[a];
    float l = (c[a] - h - o[a]) * inv;
    float u = (c[a] + h - o[a]) * inv;
    if (u < l) { float t = l; l = u; u = t; }
    if (u < lo) return 0;
    if (l > hi) return 0;
    lo = (l > lo) ? l : lo;
    hi = (u < hi) ? u : hi;
    if (lo > hi) return 0;
  }
  *t_lo = lo;
  *t_hi = hi;
  return 1;
}

/* Brute-force AABB intersection: every ray tests voxels k = 0..n-1 in index
 * order and keeps the first n_max hits. Outputs are [b, m, n_max]; idx is -1
 * and the depths 0 where there is no hit (the reference allocates zeros and
 * the kernel writes -1 into idx). points is [b, n, 3]. */
void or_aabb_intersect(int b, int n, int m, float voxelsize, int n_max,
                       const float *ray_start, const float *ray_dir, const float *points,
                       int32_t *idx, float *min_depth, float *max_depth) {
  float hv = voxelsize * 0.5f;
  for (int g = 0; g < b; ++g) {
    const float *P = points + (int64_t)g * n * 3;
    for (int j = 0; j < m; ++j) {
      int64_t r = (int64_t)g * m + j;
      const float *o = ray_start + r * 3, *d = ray_dir + r * 3;
      int32_t *I = idx + r * n_max;
      float *lo = min_depth + r * n_max, *hi = max_depth + r * n_max;
      for (int l = 0; l < n_max; ++l) { I[l] = -1; lo[l] = 0.0f; hi[l] = 0.0f; }
      int cnt = 0;
      for (int k = 0; k < n && cnt < n_max; ++k) {
        float t0, t1;
        if (or_slab(o, d, P + (int64_t)k * 3, hv, &t0, &t1) && t0 > -1.0f) {
          I[cnt] = k; lo[cnt] = t0; hi[cnt] = t1; ++cnt;
        }
      }
    }
  }
}

/* Sparse-voxel-octree intersection, restated with the reference's explicit
 * stack: pop a node, test it, emit it if it is a leaf (children[8] == 1),
 * otherwise push its existing children 0..7 (so child 7 is popped first).
 * Stops after n_max emitted leaves. The root is row n-1. The stack is capped
 * at 256 entries like the reference; returns the number of rays whose stack
 * would have overflowed (the reference asserts there). */
int or_svo_intersect(int b, int n, int m, float voxelsize, int n_max,
                     const float *ray_start, const float *ray_dir, const float *points,
                     const int32_t *children, int32_t *idx, float *min_depth, float *max_depth) {
  float hv = voxelsize * 0.5f;
  int overflow = 0;
  for (int g = 0; g < b; ++g) {
    const float *P = points + (int64_t)g * n * 3;
    const int32_t *C = children + (int64_t)g * n * 9;
    for (int j = 0; j < m; ++j) {
      int64_t r = (int64_t)g * m + j;
      const float *o = ray_start + r * 3, *d = ray_dir + r * 3;
      int32_t *I = idx + r * n_max;
      float *lo = min_depth + r * n_max, *hi = max_depth + r * n_max;
      for (int l = 0; l < n_max; ++l) { I[l] = -1; lo[l] = 0.0f; hi[l] = 0.0f; }
      int stack[256];
      int ptr = 0, cnt = 0;
      stack[0] = n - 1;
      while (ptr > -1 && cnt < n_max) {
        int k = stack[ptr--];
        float t0, t1;
        float half = hv * (float)C[(int64_t)k * 9 + 8];
        if (!(or_slab(o, d, P + (int64_t)k * 3, half, &t0, &t1) && t0 > -1.0f)) continue;
        if (C[(int64_t)k * 9 + 8] == 1) {
          I[cnt] = k; lo[cnt] = t0; hi[cnt] = t1; ++cnt;
          continue;
        }
        for (int u = 0; u < 8; ++u) {
          int ch = C[(int64_t)k * 9 + u];
          if (ch > -1) {
            if (ptr + 1 >= 256) { overflow++; ptr = -1; break; }
            stack[++ptr] = ch;
          }
        }
      }
    }
  }
  return overflow;
}

/* Ball intersection (ray vs sphere of `radius` around each point); the first
 * n_max hits in point order. Kept for API completeness (no caller in the
 * reference). The reference squares the projection with pow(x, 2); the
 * oracle and the product use x * x, so parity for this op is to a tolerance. */
void or_ball_intersect(int b, int n, int m, float radius, int n_max,
                       const float *ray_start, const float *ray_dir, const float *points,
                       int32_t *idx, float *min_depth, float *max_depth) {
  float r2max = radius * radius;
  for (int g = 0; g < b; ++g) {
    const float *P = points + (int64_t)g * n * 3;
    for (int j = 0; j < m; ++j) {
      int64_t r = (int64_t)g * m + j;
      const float *o = ray_start + r * 3, *d = ray_dir + r * 3;
      int32_t *I = idx + r * n_max;
      float *lo = min_depth + r * n_max, *hi = max_depth + r * n_max;
      for (int l = 0; l < n_max; ++l) { I[l] = -1; lo[l] = 0.0f; hi[l] = 0.0f; }
      int cnt = 0;
      for (int k = 0; k < n && cnt < n_max; ++k) {
        float x = P[k * 3 + 0] - o[0], y = P[k * 3 + 1] - o[1], z = P[k * 3 + 2] - o[2];
        /* nvcc contracts x*x + y*y + z*z into two FMAs: fma(z,z,fma(y,y,x*x)) */
        float d2 = fmaf(z, z, fmaf(y, y, x * x));
        float proj = fmaf(z, d[2], fmaf(y, d[1], x * d[0]));
        float p2 = proj * proj;
        float r2 = d2 - p2;
        if (r2 < r2max) {
          float depth = sqrtf(p2);
          float blur = sqrtf(r2max - r2);
          I[cnt] = k; lo[cnt] = depth - blur; hi[cnt] = depth + blur; ++cnt;
        }
      }
    }
  }
}

/* Ray-triangle test (Moller-Trumbore with a `blur` margin on the
 * barycentrics) with the reference's float3 helpers as nvcc contracts them
 * (fairnr/clib/include/cutil_math.h:404-413; the first product of a sum is
 * the one fused): dot = (x*x' + y*y') + z*z' -> fma(z, z', fma(x, x', y*y')),
 * cross components a*b - c*d -> fma(a, b, -(c*d)). Checked bit for bit
 * against the reference's kernel body compiled for the CPU with contraction
 * on. Returns t > 0 on a hit (with u, v), else t = -1. 1/det is IEEE (the
 * reference's __fdividef is approximate). */
static float or_dot(const float a[3], const float b[3]) {
  return fmaf(a[2], b[2], fmaf(a[0], b[0], a[1] * b[1]));
}
static void or_cross(const float a[3], const float b[3], float c[3]) {
  c[0] = fmaf(a[1], b[2], -(a[2] * b[1]));
  c[1] = fmaf(a[2], b[0], -(a[0] * b[2]));
  c[2] = fmaf(a[0], b[1], -(a[1] * b[0]));
}
static float or_tri(const float o[3], const float d[3], const float *v, float blur, float *u_out,
                    float *v_out) {
  float e1[3], e2[3], ov[3], p[3], q[3];
  for (int k = 0; k < 3; ++k) {
    e1[k] = v[3 + k] - v[k];
    e2[k] = v[6 + k] - v[k];
    ov[k] = o[k] - v[k];
  }
  or_cross(d, e2, p);
  float det = or_dot(e1, p);
  det = 1.0f / det;
  float u = or_dot(ov, p) * det;
  if ((u < 0.0f - blur) || (u > 1.0f + blur)) return -1.0f;
  or_cross(ov, e1, q);
  float w = or_dot(d, q) * det;
  if ((w < 0.0f - blur) || (w > 1.0f + blur)) return -1.0f;
  if (((u + w) < 0.0f - blur) || ((u + w) > 1.0f + blur)) return -1.0f;
  *u_out = u;
  *v_out = w;
  return or_dot(e2, q) * det;
}

/* Triangle intersection (mesh encoder): per ray, the first n_max triangles
 * with t > 0 in face order, kept sorted by depth by insertion (a new hit
 * moves past every stored one with a depth <= its own). Layout: faces
 * [b, n, 9] (three vertices), idx [b, m, n_max] (-1 pad), depth
 * [b, m, n_max * 3] = per hit (t, min offset, max offset) with the offsets
 * -cagesize / +cagesize at the ends of the list and otherwise minus / plus
 * min(cagesize, half the gap to the neighbouring hit) (0 where unused), uv
 * [b, m, n_max * 2]. */
void or_triangle_intersect(int b, int n, int m, float cagesize, float blur, int n_max,
                           const float *ray_start, const float *ray_dir, const float *faces,
                           int32_t *idx, float *depth, float *uv) {
  for (int g = 0; g < b; ++g) {
    const float *F = faces + (int64_t)g * n * 9;
    for (int j = 0; j < m; ++j) {
      int64_t r = (int64_t)g * m + j;
      const float *o = ray_start + r * 3, *d = ray_dir + r * 3;
      int32_t *I = idx + r * n_max;
      float *D = depth + r * n_max * 3, *UV = uv + r * n_max * 2;
      for (int l = 0; l < n_max; ++l) {
        I[l] = -1;
        D[3 * l] = D[3 * l + 1] = D[3 * l + 2] = 0.0f;
        UV[2 * l] = UV[2 * l + 1] = 0.0f;
      }
      int cnt = 0;
      for (int k = 0; k < n && cnt < n_max; ++k) {
        float u, w;
        float t = or_tri(o, d, F + (int64_t)k * 9, blur, &u, &w);
        if (!(t > 0.0f)) continue;
        int ki = k;
        for (int l = 0; l < cnt; ++l) {
          if (t < D[3 * l]) {
            int ti = I[l]; I[l] = ki; ki = ti;
            float tt = D[3 * l]; D[3 * l] = t; t = tt;
            float tu = UV[2 * l]; UV[2 * l] = u; u = tu;
            float tv = UV[2 * l + 1]; UV[2 * l + 1] = w; w = tv;
          }
        }
        I[cnt] = ki; D[3 * cnt] = t; UV[2 * cnt] = u; UV[2 * cnt + 1] = w;
        ++cnt;
      }
      /* fairnr/clib/src/intersect_gpu.cu:331-345 (.5 * float is exact) */
      for (int l = 0; l < cnt; ++l) {
        D[3 * l + 1] = (l == 0) ? -cagesize : -fminf(cagesize, 0.5f * (D[3 * l] - D[3 * l - 3]));
        D[3 * l + 2] = (l == cnt - 1) ? cagesize : fminf(cagesize, 0.5f * (D[3 * l + 3] - D[3 * l]));
      }
    }
  }
}

/* Uniform sampling (three-way merge of interval starts, interval ends and
 * jittered uniform steps, then midpoints kept only inside a voxel).
 * Layout: pts_idx/min/max [b, num_rays, max_hits], noise and outputs
 * [b, num_rays, max_steps]. Outputs are fully written (idx -1, depth/dist 0
 * where unused beyond the kernel's own writes, like the reference allocation). */
void or_uniform_sampling(int b, int num_rays, int max_hits, int max_steps, float step_size,
                         const int32_t *pts_idx, const float *min_depth, const float *max_depth,
                         const float *noise, int32_t *s_idx, float *s_depth, float *s_dist) {
  for (int g = 0; g < b; ++g) {
    for (int j = 0; j < num_rays; ++j) {
      int64_t r = (int64_t)g * num_rays + j;
      const int32_t *I = pts_idx + r * max_hits;
      const float *lo = min_depth + r * max_hits, *hi = max_depth + r * max_hits;
      const float *U = noise + r * max_steps;
      int32_t *SI = s_idx + r * max_steps;
      float *SD = s_depth + r * max_steps, *SS = s_dist + r * max_steps;
      for (int l = 0; l < max_steps; ++l) { SI[l] = -1; SD[l] = 0.0f; SS[l] = 0.0f; }

      int s = 0, ucur = 0, umin = 0, umax = 0;
      float lmin = 0.0f, lmax = 0.0f, cur = 0.0f;
      for (;;) {
        if (umax == max_hits || ucur == max_steps || I[umax] == -1) break;
        /* The reference writes past the row when s reaches max_steps (the
         * wrapper sizes max_steps so that this should not happen); stop. */
        if (s >= max_steps) break;
        lmin = (umin < max_hits) ? lo[umin] : 10000.0f;
        lmax = (umax < max_hits) ? hi[umax] : 10000.0f;
        if (ucur < max_steps) cur = fmaf((float)ucur + U[ucur], step_size, lo[0]);
        if (lmax <= cur && lmax <= lmin) {
          SD[s] = lmax; SI[s] = I[umax]; umax++; s++; continue;
        }
        if (cur <= lmin && cur <= lmax) {
          /* umin == 0 only when the jitter is exactly 0; the reference then
           * reads the element before the ray's row (previous ray's last id). */
          int64_t off = r * max_hits + umin - 1;
          SD[s] = cur; SI[s] = (off >= 0) ? pts_idx[off] : -1; ucur++; s++; continue;
        }
        if (lmin <= cur && lmin <= lmax) {
          SD[s] = lmin; SI[s] = I[umin]; umin++; s++; continue;
        }
        /* NaN inputs: none of the branches is taken and the reference spins
         * forever; the oracle stops instead. */
        break;
      }

      int step = 0;
      umin = 0; umax = 0;
      for (ucur = 0; ucur < max_steps - 1; ucur++) {
        if (SI[ucur + 1] == -1) break;
        float l = SD[ucur], rr = SD[ucur + 1];
        SD[ucur] = (l + rr) * 0.5f;
        SS[ucur] = rr - l;
        if (umin < max_hits && SD[ucur] >= lo[umin] && I[umin] > -1) umin++;
        if (umax < max_hits && SD[ucur] >= hi[umax] && I[umax] > -1) umax++;
        if (umax == max_hits || I[umax] == -1) break;
        if (umin - 1 == umax && SS[ucur] > 0) {
          SD[step] = SD[ucur]; SS[step] = SS[ucur]; SI[step] = SI[ucur]; step++;
        }
      }
      for (int q = step; q < max_steps; ++q) SI[q] = -1;
    }
  }
}

/* Inverse-CDF sampling over the hit intervals of each ray.
 * Layout as above plus probs [b, num_rays, max_hits] and steps [b, num_rays].
 *
 * Two reads of the reference leave the ray's own row, and both depend on how
 * the caller blocked the rays:
 *  - the tail loop tests "is the next bin empty" on pts_idx[curr_bin] of the
 *    block's FIRST ray, not the current ray (fairnr/clib/src/sample_gpu.cu:194);
 *  - when the tail loop runs with curr_bin == max_hits it reads
 *    pts_idx[H + max_hits], the first id of the NEXT row in memory
 *    (fairnr/clib/src/sample_gpu.cu:189).
 * `tail_row[r]` and `next_row[r]` (flattened over b*num_rays) name those
 * rows; next_row -1 means "past the end of the tensor" (read as -1 here; the
 * reference reads whatever lies there). NULL means the raw kernel layout:
 * row 0 of the ray's block and row r+1. */
void or_inverse_cdf(int b, int num_rays, int max_hits, int max_steps, float fixed_step_size,
                    const int32_t *pts_idx, const float *min_depth, const float *max_depth,
                    const float *noise, const float *probs, const float *steps,
                    const int64_t *tail_row, const int64_t *next_row,
                    int32_t *s_idx, float *s_depth, float *s_dist) {
  int64_t total = (int64_t)b * num_rays;
  for (int64_t r = 0; r < total; ++r) {
    int64_t g = r / num_rays;
    const int32_t *I = pts_idx + r * max_hits;
    const int32_t *I0 = pts_idx + (tail_row ? tail_row[r] : g * num_rays) * max_hits;
    int64_t nxt = next_row ? next_row[r] : ((r + 1 < total) ? r + 1 : -1);
    const float *lo = min_depth + r * max_hits, *hi = max_depth + r * max_hits;
    const float *pr = probs + r * max_hits;
    const float *U = noise + r * max_steps;
    int32_t *SI = s_idx + r * max_steps;
    float *SD = s_depth + r * max_steps, *SS = s_dist + r * max_steps;
    for (int l = 0; l < max_steps; ++l) { SI[l] = -1; SD[l] = 0.0f; SS[l] = 0.0f; }

    int bin = 0, s = 0;
    float cmin = lo[0], cmax = hi[0];
    float cdf_lo = 0.0f, cdf_hi = pr[0];
    /* `1.0 / steps[j]` is a double division rounded to float */
    float step_size = (float)(1.0 / (double)steps[r]);
    float z_low = cmin;
    int total_steps = (int)ceilf(steps[r]);
    int done = 0;
    if (fixed_step_size > 0.0f) step_size = fixed_step_size;

    for (int st = 0; st < total_steps; ++st) {
      float cdf = ((float)st + U[st]) * step_size;
      while (cdf > cdf_hi) {
        SI[s] = I[bin];
        SS[s] = cmax - z_low;
        SD[s] = (cmax + z_low) * 0.5f;
        bin++; s++;
        if (bin >= max_hits || I[bin] == -1) { done = 1; break; }
        cmin = lo[bin]; cmax = hi[bin];
        cdf_lo = cdf_hi;
        cdf_hi = cdf_hi + pr[bin];
        z_low = cmin;
      }
      if (done) break;
      float u = (cdf - cdf_lo) / (cdf_hi - cdf_lo);
      float z = fmaf(u, cmax - cmin, cmin);
      SI[s] = I[bin];
      SS[s] = z - z_low;
      SD[s] = (z + z_low) * 0.5f;
      z_low = z; s++;
    }
    /* The reference's tail loop runs even after `done` (its `~done` is always
     * true), so a finished ray re-emits its last partial segment once. */
    while (z_low < cmax) {
      int32_t id;
      if (bin < max_hits) id = I[bin];
      else id = (nxt >= 0) ? pts_idx[nxt * max_hits] : -1;
      SI[s] = id;
      SS[s] = cmax - z_low;
      SD[s] = (cmax + z_low) * 0.5f;
      bin++; s++;
      if (bin >= max_hits || I0[bin] == -1) break;
      cmin = lo[bin]; cmax = hi[bin];
      z_low = cmin;
    }
  }
}

/* ---------------------------------------------------------------------- */
/* Octree build (EasyOctree): insert every point from the root, creating the
 * missing internal nodes on the way, then number the nodes breadth first.
 * Leaves keep their point index 0..V-1; internal nodes get decreasing ids
 * from n_nodes-1 (root) in BFS order. centers are truncated to int. */

typedef struct OrNode {
  int depth;      /* -1 for leaves */
  int index;
  float c[3];     /* centre; leaves hold the integer point */
  int child[8];   /* index into the node pool, -1 if absent */
} OrNode;

typedef struct OrPool { OrNode *v; int n, cap; } OrPool;

static int or_pool_new(OrPool *p, const float c[3], int depth, int index) {
  if (p->n == p->cap) {
    p->cap = p->cap ? p->cap * 2 : 1024;
    p->v = (OrNode *)realloc(p->v, (size_t)p->cap * sizeof(OrNode));
  }
  OrNode *x = &p->v[p->n];
  x->depth = depth; x->index = index;
  x->c[0] = c[0]; x->c[1] = c[1]; x->c[2] = c[2];
  for (int i = 0; i < 8; ++i) x->child[i] = -1;
  return p->n++;
}

/* Returns the number of nodes; writes at most max_nodes rows of
 * centers [.,3] int32 and children [.,9] int32. Returns -1 on a bad
 * input (point outside the root cube) and -2 if max_nodes is too small. */
int64_t or_build_octree(const float center[3], const int64_t *points, int64_t npts, int depth,
                        int32_t *centers, int32_t *children, int64_t max_nodes) {
  OrPool pool = {0, 0, 0};
  int root = or_pool_new(&pool, center, depth, -1);
  for (int64_t k = 0; k < npts; ++k) {
    float pt[3] = {(float)points[k * 3 + 0], (float)points[k * 3 + 1], (float)points[k * 3 + 2]};
    int cur = root;
    for (;;) {
      OrNode *p = &pool.v[cur];
      int dx = pt[0] > p->c[0], dy = pt[1] > p->c[1], dz = pt[2] > p->c[2];
      int ci = dx + 2 * dy + 4 * dz;
      if (p->depth == 0) {
        int leaf = or_pool_new(&pool, pt, -1, (int)k);
        pool.v[cur].child[ci] = leaf;
        break;
      }
      if (p->child[ci] < 0) {
        float len = (float)(1 << (p->depth - 1));
        float nc[3] = {p->c[0] + (float)(2 * dx - 1) * len,
                       p->c[1] + (float)(2 * dy - 1) * len,
                       p->c[2] + (float)(2 * dz - 1) * len};
        int pd = p->depth;
        int nn = or_pool_new(&pool, nc, pd - 1, -1);
        pool.v[cur].child[ci] = nn;
      }
      cur = pool.v[cur].child[ci];
    }
  }
  /* count: every node reachable from the root (overwritten leaves are not) */
  int64_t total = 0, terminal = 0;
  int *queue = (int *)malloc((size_t)pool.n * sizeof(int));
  int qh = 0, qt = 0;
  queue[qt++] = root;
  while (qh < qt) {
    OrNode *x = &pool.v[queue[qh++]];
    total++;
    if (x->depth == -1) terminal++;
    for (int i = 0; i < 8; ++i) if (x->child[i] >= 0) queue[qt++] = x->child[i];
  }
  if (total > max_nodes) { free(queue); free(pool.v); return -2; }
  for (int64_t i = 0; i < total * 3; ++i) centers[i] = 0;
  for (int64_t i = 0; i < total * 9; ++i) children[i] = -1;
  int64_t node_idx = total - 1;
  pool.v[root].index = (int)node_idx;
  qh = 0; qt = 0;
  queue[qt++] = root;
  while (qh < qt) {
    OrNode *x = &pool.v[queue[qh++]];
    for (int i = 0; i < 8; ++i) {
      int c = x->child[i];
      if (c < 0) continue;
      OrNode *y = &pool.v[c];
      if (y->depth > -1) { node_idx--; y->index = (int)node_idx; }
      queue[qt++] = c;
      children[(int64_t)x->index * 9 + i] = y->index;
    }
    children[(int64_t)x->index * 9 + 8] = 1 << (x->depth + 1);
    for (int a = 0; a < 3; ++a) centers[(int64_t)x->index * 3 + a] = (int32_t)x->c[a];
  }
  free(queue);
  free(pool.v);
  return (node_idx == terminal) ? total : -3;
}
