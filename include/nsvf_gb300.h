/*
 * nsvf_gb300 -- C ABI of the GB300-native (sm_103a) sparse-voxel rendering
 * hot path of NSVF (facebookresearch/NSVF, package `fairnr`).
 *
 * Every entry point takes plain device pointers, sizes and a CUDA stream
 * (passed as `void *`, a cudaStream_t), launches asynchronously on that
 * stream, allocates nothing unless stated, and returns an int status
 * (NSVF_OK or a negative NSVF_ERR_*). None of them exits the process: the
 * reference's CUDA_CHECK_ERRORS calls exit(-1) on a launch error
 * (fairnr/clib/include/cuda_utils.h:35-44).
 *
 * Layouts are row-major and contiguous; "[b, m, 3]" means b*m*3 elements.
 *
 * Floating point: geometry ops compute in FP32 with the reference's
 * operation order and its fused multiply-adds (nvcc contracts `a + b * c` by
 * default); the one deliberate difference is the ray reciprocal 1/dir, which
 * the reference takes with the approximate __fdividef and this library with
 * the correctly rounded __frcp_rn, so results are reproducible bit for bit on
 * a CPU.
 */
#ifndef NSVF_GB300_H
#define NSVF_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NSVF_OK 0
#define NSVF_ERR_INVALID (-1)   /* bad sizes or null pointers */
#define NSVF_ERR_CUDA (-2)      /* a CUDA launch or API call failed */
#define NSVF_ERR_OCTREE (-3)    /* malformed octree (host validation) */
#define NSVF_ERR_CAPACITY (-4)  /* an output buffer is too small */

/* Human-readable text for a status code. */
const char *nsvf_status_string(int status);

/* Number of kernels this library has launched in this process (all
 * devices, all streams); for profiling and launch accounting. */
long long nsvf_launch_count(void);

/* ------------------------------------------------------------------------ */
/* Ray-voxel intersection (fairnr/clib/include/intersect.h:10-17)            */

/* aabb_intersect: replaces `aabb_intersect(ray_start, ray_dir, points,
 * voxelsize, n_max)` (fairnr/clib/src/intersect.cpp:49-75,
 * fairnr/clib/src/intersect_gpu.cu:125-167).
 * ray_start, ray_dir [b, m, 3]; points [b_pts, n, 3] with b_pts == b or 1
 * (1 = one voxel set shared by all b ray batches; the reference copies it b
 * times). Each ray tests voxels 0..n-1 in index order and keeps its first
 * n_max hits. Outputs [b, m, n_max]: idx (int32, -1 = none), min_depth and
 * max_depth (FP32, 0 = none). */
int nsvf_aabb_intersect(int b, int b_pts, int n, int m, float voxelsize, int n_max,
                        const float *ray_start, const float *ray_dir, const float *points,
                        int32_t *idx, float *min_depth, float *max_depth, void *stream);

/* svo_intersect: replaces `svo_intersect(ray_start, ray_dir, points,
 * children, voxelsize, n_max)` (fairnr/clib/src/intersect.cpp:84-112,
 * fairnr/clib/src/intersect_gpu.cu:170-237).
 * points [b_pts, n, 3] node centres, children [b_pts, n, 9] int32 (8 child
 * ids or -1, then the node size in leaf units: 1 for a leaf); the root is row
 * n-1. Rays traverse the octree depth first, visiting children 7..0, and keep
 * the first n_max leaves hit, in that order. Outputs as aabb_intersect.
 * `workspace` is device memory of nsvf_svo_workspace_bytes(b_pts, n) bytes,
 * 16-byte aligned, used for a packed copy of the octree (it may be reused for
 * the next call only after this call's kernels have finished). `err` (device
 * int, may be NULL) gets bit 0 set if the octree is malformed (a child id
 * outside [0, n), a cycle, or deeper than 36 levels); such rays stop early
 * instead of reading out of bounds (the reference asserts or faults). */
int64_t nsvf_svo_workspace_bytes(int b_pts, int n);
int nsvf_svo_intersect(int b, int b_pts, int n, int m, float voxelsize, int n_max,
                       const float *ray_start, const float *ray_dir, const float *points,
                       const int32_t *children, int32_t *idx, float *min_depth,
                       float *max_depth, int32_t *err, void *workspace, void *stream);

/* svo_pack: writes the packed copy of ONE octree (points [n, 3], children
 * [n, 9]) that the sorted traversal reads into `workspace`
 * (nsvf_svo_workspace_bytes(1, n) bytes, 16-byte aligned), so that
 * nsvf_svo_intersect_grid can reuse it across calls. The packing step of
 * fairnr/clib/__init__.py:101-111 (the reference copies the octree once per
 * ray block on every call). */
int nsvf_svo_pack(int n, float voxelsize, const float *points, const int32_t *children,
                  void *workspace, void *stream);

/* svo_grid_build: HOST function (host pointers, no GPU needed). Builds the
 * leaf-grid form of ONE octree (points [n, 3], children [n, 9], both host
 * memory) for nsvf_svo_intersect_grid: the leaves' FP32 centres as per-axis
 * grid lines, a 4x4x4-brick occupancy bitmap with prefix counts, each leaf's
 * rank in the depth-first visiting order of
 * fairnr/clib/src/intersect_gpu.cu:200-235, and a flag on leaves whose
 * ancestors' FP32 faces do not all enclose their own. Writes the blob into
 * `grid` (`capacity` bytes); `*bytes` (may be NULL) gets its size. Returns
 * NSVF_ERR_CAPACITY with `*bytes` set when `grid` is NULL or too small (call
 * once to size, once to fill), and NSVF_ERR_OCTREE when the tree is not in
 * leaf-grid form: a child id >= n, a node reached twice, a node deeper than
 * 15 levels, a size < 1, two different centres on one grid line, two leaves
 * in one cell, or more than 65,536 grid lines on an axis. Such trees go
 * through nsvf_svo_intersect_sorted, which reports the malformed ones. Copy
 * the blob to device memory (16-byte aligned) for the intersection. */
int nsvf_svo_grid_build(int n, float voxelsize, const float *points, const int32_t *children,
                        void *grid, int64_t capacity, int64_t *bytes);
/* out[6] = grid lines x, y, z, leaves, flagged leaves, nodes of a HOST copy
 * of a blob. */
int nsvf_svo_grid_info(const void *grid_host, int32_t *out);
/* Device bytes of the ray list nsvf_svo_intersect_grid needs for `rays`. */
int64_t nsvf_svo_grid_list_bytes(int64_t rays);

/* svo_intersect_grid: the outputs of nsvf_svo_intersect_sorted (b = 1, one
 * octree: rays [rays, 3]; idx/min_depth/max_depth [rays, n_max], hits
 * [rays]), bit for bit, replacing svo_intersect + the encoder's sort
 * (fairnr/clib/src/intersect_gpu.cu:170-237, fairnr/modules/encoder.py:
 * 518-524) by a sweep of each ray across the grid of leaf cells, one thread
 * per ray, in order of depth. `grid` is the device copy of the
 * nsvf_svo_grid_build blob, `info` (HOST int32[6]) its nsvf_svo_grid_info,
 * `packed` the nsvf_svo_pack workspace of the
 * same octree, `list_ws` nsvf_svo_grid_list_bytes(rays) bytes of device
 * scratch (16-byte aligned). The hits of a ray past its first n_max go to
 * an overflow block there (32,768 blocks at most), and an overflow pass (a
 * warp per ray) keeps, like the search, the first n_max leaves in visiting
 * order. Rays the sweep leaves to the depth-first search are listed there
 * and traversed by it in a last launch: rays with a zero direction
 * component, with a hit beyond depth 10000, with more than n_max + 64 hits,
 * or past the last overflow block. n_max <= 128. Calls that share `list_ws` must not overlap on the
 * GPU. */
int nsvf_svo_intersect_grid(int64_t rays, int n, float voxelsize, int n_max,
                            const float *ray_start, const float *ray_dir, const float *points,
                            const int32_t *children, const void *grid, const int32_t *info,
                            const void *packed, void *list_ws, int32_t *idx, float *min_depth,
                            float *max_depth, uint8_t *hits, int32_t *err, void *stream);
/* svo_intersect_grid_rows: nsvf_svo_intersect_grid with pad_rows = 1; with
 * pad_rows = 0 the rows of rays the sweep finishes are not padded: a hit
 * ray's row ends with one -1 after its last hit (when it has fewer than
 * n_max), a missed ray's row is not written (hits[r] = 0), and slots past
 * the -1 keep what they held. Rows of overflow rays and of rays listed for
 * the depth-first search are complete. For readers that stop at a row's
 * first -1, such as nsvf_gather_probs: the rows' padding is most of the
 * call's writes (12 * n_max bytes per missed ray). */
int nsvf_svo_intersect_grid_rows(int64_t rays, int n, float voxelsize, int n_max,
                                 const float *ray_start, const float *ray_dir,
                                 const float *points, const int32_t *children, const void *grid,
                                 const int32_t *info, const void *packed, void *list_ws,
                                 int32_t *idx, float *min_depth, float *max_depth, uint8_t *hits,
                                 int32_t *err, int pad_rows, void *stream);

/* svo_intersect_noalloc: has no counterpart in the reference. The same
 * computation and outputs as nsvf_svo_intersect, for callers that cannot
 * allocate device memory on the call path (a real-time render loop, or a host
 * engine that pre-partitions GPU memory and passes only its own input and
 * output buffers): instead of a caller-provided workspace it uses a scratch
 * array inside this library, fixed at NSVF_NOALLOC_MAX_NODES octree nodes
 * (b_pts * n, 176 bytes each: 44 MiB, held by every GPU that loads the
 * library until the process exits). Larger octrees are rejected with
 * NSVF_ERR_CAPACITY. It allocates nothing: the first call on a device looks
 * the array's device address up (cudaGetSymbolAddress, once per device,
 * cached), so make that first call before any stream capture. The cached
 * address does not survive a device reset (cudaDeviceReset, or a primary
 * context released and created again): do not call this entry point on a
 * device after resetting it. All calls share the one array: calls that
 * overlap on the GPU (other streams, other threads) race and must be
 * serialised by the caller. */
#define NSVF_NOALLOC_MAX_NODES (1 << 18)
int nsvf_svo_intersect_noalloc(int b, int b_pts, int n, int m, float voxelsize, int n_max,
                               const float *ray_start, const float *ray_dir, const float *points,
                               const int32_t *children, int32_t *idx, float *min_depth,
                               float *max_depth, int32_t *err, void *stream);

/* svo_intersect_sorted: svo_intersect followed by the encoder's
 * post-processing (fairnr/modules/encoder.py:518-524) in the same kernel:
 * missing slots get depth 10000 (MAX_DEPTH), each ray's n_max slots are
 * sorted by min_depth (stable: ties keep traversal order), and hits[b*m]
 * (uint8) is 1 where a ray hit any voxel. n_max <= 128. */
int nsvf_svo_intersect_sorted(int b, int b_pts, int n, int m, float voxelsize, int n_max,
                              const float *ray_start, const float *ray_dir, const float *points,
                              const int32_t *children, int32_t *idx, float *min_depth,
                              float *max_depth, uint8_t *hits, int32_t *err, void *workspace,
                              void *stream);

/* triangle_intersect: replaces triangle_intersect (fairnr/clib/src/
 * intersect.cpp:120-145, kernel fairnr/clib/src/intersect_gpu.cu:238-345),
 * the mesh encoder's ray-triangle op. face_points [b_faces, n, 9] (three
 * vertices per face; b_faces 1 = shared by all b rows, where the reference
 * copies it per row). Per ray: the first n_max faces with t > 0 in face
 * order, sorted by depth (insertion; ties keep face order), idx [b, m,
 * n_max] (-1 pad), depth [b, m, 3 n_max] = per hit (t, -min(cagesize, half
 * the gap to the previous hit), +min(cagesize, half the gap to the next);
 * -/+cagesize at the ends), uv [b, m, 2 n_max] barycentrics; unused slots 0.
 * Moller-Trumbore with the reference's `blur` margin and its FP32 operation
 * sequence; 1/det correctly rounded. */
int nsvf_triangle_intersect(int b, int b_faces, int n, int m, float cagesize, float blur,
                            int n_max, const float *ray_start, const float *ray_dir,
                            const float *face_points, int32_t *idx, float *depth, float *uv,
                            void *stream);

/* ball_intersect: replaces `ball_intersect(ray_start, ray_dir, points,
 * radius, n_max)` (fairnr/clib/src/intersect.cpp:15-41). Rays vs spheres of
 * `radius` around each point; first n_max hits in point order. */
int nsvf_ball_intersect(int b, int b_pts, int n, int m, float radius, int n_max,
                        const float *ray_start, const float *ray_dir, const float *points,
                        int32_t *idx, float *min_depth, float *max_depth, void *stream);

/* ------------------------------------------------------------------------ */
/* Sample placement (fairnr/clib/include/sample.h:11-16)                     */

/* uniform_ray_sampling: replaces `uniform_ray_sampling(pts_idx, min_depth,
 * max_depth, uniform_noise, step_size, max_steps)`
 * (fairnr/clib/src/sample.cpp:23-55, fairnr/clib/src/sample_gpu.cu:15-106).
 * pts_idx/min_depth/max_depth [b, m, max_hits], noise [b, m, max_steps];
 * outputs sampled_idx (int32, -1 pad), sampled_depth, sampled_dists
 * [b, m, max_steps], fully written. `err` (device int, may be NULL) gets
 * bit 1 set if a ray needed more than max_steps slots (the reference writes
 * past its row there). */
int nsvf_uniform_ray_sampling(int b, int m, int max_hits, int max_steps, float step_size,
                              const int32_t *pts_idx, const float *min_depth,
                              const float *max_depth, const float *noise, int32_t *sampled_idx,
                              float *sampled_depth, float *sampled_dists, int32_t *err,
                              void *stream);

/* parallel_ray_sampling: the reference's back-up uniform sampler
 * (`_parallel_ray_sampling`, fairnr/clib/__init__.py:303-349, pure torch
 * there), one chunk of rows. Per row (pts_idx/min_depth/max_depth
 * [rows, max_hits], sorted hit lists with MAX_DEPTH in missing slots): steps
 * u_k = min_depth[0] + (k + j_k) * march_size, k < n_steps (j = noise
 * [rows, n_steps], or 0.5 when noise is NULL), each with the id of slot
 * #{i : min_depth_i <= u_k} - 1; the exits, entries and steps sorted
 * (ties in that order, so that at a face shared by two voxels the next
 * segment takes the entered voxel's id; the reference's torch.sort leaves
 * such ties unspecified); between consecutive depths a segment with midpoint
 * .5 (a + b), length b - a and the first depth's id, kept when it lies in one
 * voxel (#{min_depth <= mid} - 1 == #{max_depth <= mid}), not beyond the last
 * exit (MAX_DEPTH exits read as 0) and not of length 0. Writes the kept
 * segments in order into sampled_idx / sampled_depth / sampled_dists
 * [rows, out_width] (then -1 / 10000 / 0) and their number to count[rows]
 * (may be NULL). out_width >= 2 max_hits + n_steps - 1 holds every segment.
 * NSVF_ERR_CAPACITY if a row's lists exceed the shared memory (4 rows per
 * block, nsvf_parallel_sampling_smem_bytes each, 224 KB in all). */
int64_t nsvf_parallel_sampling_smem_bytes(int max_hits, int n_steps);
int nsvf_parallel_ray_sampling(int64_t rows, int max_hits, int n_steps, float march_size,
                               const int32_t *pts_idx, const float *min_depth,
                               const float *max_depth, const float *noise, int out_width,
                               int32_t *sampled_idx, float *sampled_depth, float *sampled_dists,
                               int32_t *count, void *stream);

/* inverse_cdf_sampling: replaces `inverse_cdf_sampling(pts_idx, min_depth,
 * max_depth, uniform_noise, probs, steps, fixed_step_size)`
 * (fairnr/clib/src/sample.cpp:58-96, fairnr/clib/src/sample_gpu.cu:108-202).
 * pts_idx/min_depth/max_depth/probs [rows, max_hits], steps [rows], noise
 * [rows, noise_stride] (noise_stride >= max_steps), outputs [rows, max_steps].
 * `noise` may be NULL: every jitter is then 0.5 (the reference's
 * deterministic mode fills a tensor with 0.5).
 *
 * Two reads of the reference leave the ray's row and depend on how the rays
 * were blocked into kernel launches (fairnr/clib/src/sample_gpu.cu:189, 194);
 * `layout` reproduces them:
 *   layout[0] = K (rays per block), layout[1] = chunk (rays of a block per
 *   launch), layout[2] = N (real rays; rows >= N are padding copies of row
 *   0), layout[3] = G (blocks).
 * For the raw op on [b, m, H] tensors pass {m, m, b*m, b}; for the
 * reference's InverseCDFRaySampling wrapper over N rays pass
 * {ceil(N/200), 800, N, 200} (fairnr/clib/__init__.py:234-270).
 * `max_len` (device int, may be NULL) receives atomically the largest number
 * of non -1 ids over the rows (the wrapper's truncation width); `err` bit 1
 * is set if a ray needed more than max_steps slots or noise columns. */
int nsvf_inverse_cdf_sampling(int64_t rows, int max_hits, int max_steps, int noise_stride,
                              float fixed_step_size, const int32_t *pts_idx,
                              const float *min_depth, const float *max_depth, const float *noise,
                              const float *probs, const float *steps, const int64_t layout[4],
                              int32_t *sampled_idx, float *sampled_depth, float *sampled_dists,
                              int32_t *max_len, int32_t *err, void *stream);

/* sample_count / sample_compact: the served renderer's form of the same
 * inverse-CDF walk (deterministic 0.5 jitter, the wrapper's launch layout):
 * sample_count writes count[r] = number of samples with a voxel id (not -1)
 * of each ray; with offset = exclusive prefix sum of count (rows + 1
 * entries), sample_compact writes those samples contiguously per ray, in
 * order: voxel[j] (int32), xyz_dist[j] = (o + d * t, max(dist, 0)) as float4,
 * depth[j] = t. This is exactly the list of valid samples the reference's
 * renderer evaluates (fairnr/modules/encoder.py:538-556,
 * fairnr/modules/renderer.py:86-100), without the padded [rows, M] tensors.
 * ray_start is [rows, 3] (stride 3) or one shared origin (stride 0). */
int nsvf_sample_count(int64_t rows, int max_hits, const int32_t *pts_idx, const float *min_depth,
                      const float *max_depth, const float *probs, const float *steps,
                      const int64_t layout[4], int32_t *count, void *stream);
int nsvf_sample_compact(int64_t rows, int max_hits, const int32_t *pts_idx,
                        const float *min_depth, const float *max_depth, const float *probs,
                        const float *steps, const int64_t layout[4], const float *ray_start,
                        int64_t ray_start_stride, const float *ray_dir, const int64_t *offset,
                        int32_t *voxel, float *xyz_dist, float *depth, int32_t *err,
                        void *stream);

/* ------------------------------------------------------------------------ */
/* Octree build (fairnr/clib/include/octree.h:10)                            */

/* build_octree: replaces `build_octree(center, points, depth)`
 * (fairnr/clib/src/octree.cpp:125-136). HOST function on host memory.
 * center[3] (float), points [n_points, 3] int64 (integer half-voxel
 * coordinates), depth. Writes up to `capacity` rows of centers [., 3] and
 * children [., 9] (int32) and returns the node count, or a negative status
 * (NSVF_ERR_CAPACITY if capacity is too small: call again with more room).
 * Numbering as the reference: leaves keep their point index 0..n_points-1,
 * internal nodes count down from n_nodes-1 (the root) in breadth-first order;
 * children[., 8] = 1 << (node depth + 1); centres truncated to int. */
int64_t nsvf_build_octree(const float center[3], const int64_t *points, int64_t n_points,
                          int depth, int32_t *centers, int32_t *children, int64_t capacity);

/* ------------------------------------------------------------------------ */
/* Trilinear interpolation of corner embeddings                              */

/* trilinear_embed: replaces the embedding part of SparseVoxelEncoder.forward
 * (fairnr/modules/encoder.py:578-590 with fairnr/data/geometry.py:195-200).
 * For sample s in voxel v = sampled_idx[s] (int32 or int64: idx_bytes 4|8):
 * p = (xyz[s] - centers[v]) / voxel_size + 0.5; corner k = 4*ix + 2*iy + iz
 * weighs prod_d (bit_d(k) ? p_d : 1 - p_d); emb[s] = sum_k w_k *
 * values[feats[v, k]]. xyz [n, 3], centers [n_voxels, 3], feats
 * [n_voxels, 8] (int32/int64: feat_bytes), values [n_keys, embed_dim], emb
 * [n, embed_dim], FP32; embed_dim in {4, 8, 16, 32, 64, 128}; values and emb
 * 16-byte aligned. Ids out of range are not read (emb 0, err bit 2). */
int nsvf_trilinear_embed(int64_t n_samples, int embed_dim, float voxel_size, int64_t n_voxels,
                         int64_t n_keys, const void *sampled_idx, int idx_bytes, const float *xyz,
                         const float *centers, const void *feats, int feat_bytes,
                         const float *values, float *emb, int32_t *err, void *stream);

/* Backward of trilinear_embed: grad_values [n_keys, embed_dim] (accumulated
 * with atomics; zero it first) and/or grad_xyz [n, 3] (written), either may
 * be NULL (not both). The reference gets these from autograd through its two
 * F.embedding gathers (an index_add into the embedding table). */
int nsvf_trilinear_embed_backward(int64_t n_samples, int embed_dim, float voxel_size,
                                  int64_t n_voxels, int64_t n_keys, const void *sampled_idx,
                                  int idx_bytes, const float *xyz, const float *centers,
                                  const void *feats, int feat_bytes, const float *values,
                                  const float *grad_emb, float *grad_values, float *grad_xyz,
                                  void *stream);

/* ------------------------------------------------------------------------ */
/* Compositing                                                               */

/* composite: replaces the compositing of VolumeRenderer.forward_chunk
 * (fairnr/modules/renderer.py:193-218) over [rays, max_steps] samples:
 * a_i = 1 - exp(-fe_i), T_i = exp(-sum_{j<i} fe_j), p_i = a_i T_i;
 * probs [rays, max_steps], depth [rays] = sum p_i t_i, missed = 1 - sum p_i,
 * colors [rays, 3] = sum p_i tex_i. texture [rays, max_steps, 3] and
 * sampled_depth may be NULL (their outputs are then skipped); any output may
 * be NULL. kahan != 0 carries the transmittance prefix as a compensated sum. */
int nsvf_composite(int64_t rays, int max_steps, const float *free_energy, const float *texture,
                   const float *sampled_depth, float *probs, float *depth, float *missed,
                   float *colors, int kahan, void *stream);

/* Backward of composite: gradients w.r.t. free_energy (written) and texture
 * (written, may be NULL) from the gradients of probs/depth/missed/colors
 * (each may be NULL = zero). */
int nsvf_composite_backward(int64_t rays, int max_steps, const float *free_energy,
                            const float *texture, const float *sampled_depth,
                            const float *grad_probs, const float *grad_depth,
                            const float *grad_missed, const float *grad_colors,
                            float *grad_free_energy, float *grad_texture, int kahan,
                            void *stream);

/* composite_segments: compositing of the compacted samples of the served
 * renderer plus the background fill of NSVFModel.postprocessing
 * (fairnr/models/nsvf.py:89-110). Ray r owns samples [offset[r],
 * offset[r+1]); field [n, 4] = (sigma, r, g, b) (16-byte aligned);
 * fe = relu(sigma) * dist * sigma_scale. Writes pixel[r] of out_color
 * [., 3] = sum p c + missed * bg, out_depth = sum p t + missed * bg_depth
 * and out_missed. */
int nsvf_composite_segments(int64_t rays, const int64_t *offset, const float *field,
                            const float *xyz_dist, const float *depth, const int64_t *pixel,
                            float sigma_scale, const float bg[3], float bg_depth,
                            float *out_color, float *out_depth, float *out_missed, int kahan,
                            void *stream);

/* ------------------------------------------------------------------------ */
/* Synchronisation-free chunk chain (served rendering under CUDA graphs)     */

/* pinhole_rays: rays of `n` pixels of a pinhole frame from 18 camera floats
 * in device memory: origin[3], camera-to-world rotation R[3][3] (row-major,
 * columns right/down/forward), focal, cx, cy, width, first pixel, pixel
 * count. Ray t = pixel first + t (row-major), direction normalize(R ((j + .5
 * - cx) / f, (i + .5 - cy) / f, 1)); rays t >= count point away from the
 * scene. The frame-to-ray step of the reference's reader
 * (fairnr/modules/reader.py:92-119, fairnr/data/geometry.py:116-122). */
int nsvf_pinhole_rays(int64_t n, const float *cam, float *ray_start, float *ray_dir,
                      void *stream);

/* pinhole_rays_multi: one serving chunk of n rays made of several pixel
 * ranges, possibly of different frames: segment s < min(*n_seg, max_seg)
 * (n_seg on the device) is cams[s] (18 floats as nsvf_pinhole_rays, its
 * first pixel and pixel count included) and takes the next cams[s][17] rays
 * of the chunk; rays past the last segment point away from the scene. */
int nsvf_pinhole_rays_multi(int64_t n, int max_seg, const int32_t *n_seg, const float *cams,
                            float *ray_start, float *ray_dir, void *stream);

/* piece_rows: the hit-row range of every segment of such a chunk, for the
 * piece-aware sampling entry points: with scan (int32 [n]) the inclusive
 * prefix sum of the chunk's hit flags, piece_rows[s + 1] = hit rows of
 * segments 0..s (max_seg + 1 entries, int64; segments past *n_seg empty). */
int nsvf_piece_rows(int max_seg, const int32_t *n_seg, const float *cams, int64_t n,
                    const int32_t *scan, int64_t *piece_rows, void *stream);

/* camera_rays: n rays in the reference's camera convention, the eval path of
 * ImageReader (fairnr/modules/reader.py:92-119) with get_uv
 * (fairnr/data/data_utils.py:57-65) and get_ray_direction
 * (fairnr/data/geometry.py:116-122). cam (device, 20 floats) = fx, fy, cx,
 * cy, inv_RT (3 x 4 camera-to-world, row-major), W / w, H / h (an H x W
 * image read at h x w), w, first pixel. Ray t is pixel first + t of the
 * w-wide grid, row-major, at integer pixel coordinates scaled to the full
 * image. ray_start[n, 3] = inv_RT's translation, ray_dir[n, 3] =
 * (rt - ray_start) / (|rt - ray_start| + 1e-8) with rt the pixel's point at
 * depth 1. */
int nsvf_camera_rays(int64_t n, const float *cam, float *ray_start, float *ray_dir,
                     void *stream);

/* compact_hits: given hits[n] (uint8) and scan = their inclusive prefix sum
 * (int32), writes the hit rays' indices in order to pix and their number to
 * *n_hit (both on the device). */
int nsvf_compact_hits(int64_t n, const uint8_t *hits, const int32_t *scan, int64_t *pix,
                      int64_t *n_hit, void *stream);

/* ray_probs: the sampling distribution of NSVFModel.intersecting
 * (fairnr/models/nsvf.py:65-74) for rows [rows, max_hits] of sorted hit
 * lists: d_k = max_depth_k - min_depth_k on hit slots (idx != -1), else 0;
 * tot = d_0 + d_1 + ... added in slot order in FP32 (the order of a plain
 * loop; torch's reduction order is unspecified and differs between builds
 * and devices); probs [rows, max_hits] = d / tot; steps [rows] = tot /
 * step_size. Rows without hits get 0 / 0 = NaN probs and 0 steps, as the
 * reference's division does. Any max_hits. */
int nsvf_ray_probs(int64_t rows, int max_hits, float step_size, const int32_t *idx,
                   const float *min_depth, const float *max_depth, float *probs, float *steps,
                   void *stream);

/* gather_probs: for rows i < *n_hit, copies the sorted hit list of ray pix[i]
 * ([., max_hits] idx/min/max) and builds its sampling distribution exactly as
 * nsvf_ray_probs does (same sum order, same roundings), so the served chain
 * samples exactly the drop-in path's samples. A row is read up to its first
 * -1 (rows of nsvf_svo_intersect_grid_rows without padding); the copies are
 * padded with id -1 and depths 10000 either way. */
int nsvf_gather_probs(int64_t cap, const int64_t *n_hit, int max_hits, float step_size,
                      const int64_t *pix, const int32_t *idx, const float *min_depth,
                      const float *max_depth, int32_t *out_idx, float *out_min, float *out_max,
                      float *probs, float *steps, void *stream);

/* sample_count_dev / sample_compact_dev: nsvf_sample_count /
 * nsvf_sample_compact with the row count *n_rows_dev read on the device
 * (rows past it: count 0) and the reference wrapper's layout for that many
 * rows; ray_index (may be NULL) maps row i to its ray's origin/direction;
 * samples past sample_cap are not written (err bit 1). */
int nsvf_sample_count_dev(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                          const int32_t *pts_idx, const float *min_depth, const float *max_depth,
                          const float *probs, const float *steps, int32_t *count, void *stream);
int nsvf_sample_compact_dev(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                            const int32_t *pts_idx, const float *min_depth,
                            const float *max_depth, const float *probs, const float *steps,
                            const float *ray_start, int64_t ray_start_stride,
                            const float *ray_dir, const int64_t *ray_index,
                            const int64_t *offset, int64_t sample_cap, int32_t *voxel,
                            float *xyz_dist, float *depth, int32_t *err, void *stream);

/* sample_count_pieces / sample_compact_pieces: nsvf_sample_count_dev /
 * nsvf_sample_compact_dev for rows made of independent pieces: piece p
 * owns rows [piece_rows[p], piece_rows[p + 1]) (max_pieces + 1 ascending
 * entries, device memory; rows past the last entry belong to the last
 * piece), and each piece gets the reference wrapper's launch layout for its
 * own row count, so a piece's samples are the same whatever else shares the
 * launch. max_pieces 0: one piece (the _dev behaviour). */
int nsvf_sample_count_pieces(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                             const int32_t *pts_idx, const float *min_depth,
                             const float *max_depth, const float *probs, const float *steps,
                             const int64_t *piece_rows, int max_pieces, int32_t *count,
                             void *stream);
int nsvf_sample_compact_pieces(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                               const int32_t *pts_idx, const float *min_depth,
                               const float *max_depth, const float *probs, const float *steps,
                               const int64_t *piece_rows, int max_pieces,
                               const float *ray_start, int64_t ray_start_stride,
                               const float *ray_dir, const int64_t *ray_index,
                               const int64_t *offset, int64_t sample_cap, int32_t *voxel,
                               float *xyz_dist, float *depth, int32_t *err, void *stream);

/* sample_scan_compact_dev / _pieces: nsvf_sample_count_dev (or _pieces),
 * the exclusive prefix sum of the counts into offset, and
 * nsvf_sample_compact_dev (or _pieces) in one pass. Blocks of 4 rows take
 * their rows in ticket order and find their first sample by a look-back over
 * the earlier blocks' published counts. The outputs are those of the three
 * steps: the same samples at the same positions, offset[r] for r < *n_rows_dev
 * and the total at offset[*n_rows_dev] and offset[rows_cap] (entries in
 * between are not written). scan_ws: device workspace of
 * nsvf_sample_scan_bytes(rows_cap) bytes, 8-byte aligned, zeroed by the call
 * on the stream (NSVF_ERR_CAPACITY if smaller). Rows with max_hits > 128 are
 * refused (NSVF_ERR_INVALID): use the two-pass entry points. A look-back
 * that waits too long sets err bit 8. Replaces the count and compaction
 * launches of the served chain's sampling (fairnr/clib/src/sample_gpu.cu:
 * 108-202 for one ray's samples). */
int64_t nsvf_sample_scan_bytes(int64_t rows_cap);
int nsvf_sample_scan_compact_dev(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                                 const int32_t *pts_idx, const float *min_depth,
                                 const float *max_depth, const float *probs, const float *steps,
                                 const float *ray_start, int64_t ray_start_stride,
                                 const float *ray_dir, const int64_t *ray_index, int64_t *offset,
                                 int64_t sample_cap, int32_t *voxel, float *xyz_dist, float *depth,
                                 void *scan_ws, int64_t scan_ws_bytes, int32_t *err,
                                 void *stream);
int nsvf_sample_scan_compact_pieces(int64_t rows_cap, const int64_t *n_rows_dev, int max_hits,
                                    const int32_t *pts_idx, const float *min_depth,
                                    const float *max_depth, const float *probs,
                                    const float *steps, const int64_t *piece_rows, int max_pieces,
                                    const float *ray_start, int64_t ray_start_stride,
                                    const float *ray_dir, const int64_t *ray_index,
                                    int64_t *offset, int64_t sample_cap, int32_t *voxel,
                                    float *xyz_dist, float *depth, void *scan_ws,
                                    int64_t scan_ws_bytes, int32_t *err, void *stream);

/* composite_segments_dev: nsvf_composite_segments over *n_rays_dev rays,
 * each ray's segment [offset[r], offset[r + 1]) clamped to the sample
 * buffers' capacity sample_cap (a frame whose samples overflowed them -- the
 * sample kernels' error bit 1 -- is to be composited again with room for all
 * of them; nothing is read past the buffers). */
int nsvf_composite_segments_dev(int64_t rays_cap, const int64_t *n_rays_dev,
                                const int64_t *offset, int64_t sample_cap, const float *field,
                                const float *xyz_dist, const float *depth, const int64_t *pixel,
                                float sigma_scale, const float bg[3], float bg_depth,
                                float *out_color, float *out_depth, float *out_missed, int kahan,
                                void *stream);

/* field_samples_bf16_dev: nsvf_field_samples_bf16 on *n_samples_dev samples
 * (at most `capacity`; a larger count sets err bit 1), one persistent CTA
 * per SM. If n_outliers is not NULL, every sample lying far outside its
 * voxel (a trilinear coordinate outside [-0.5, 1.5]) is also appended to
 * outliers (int64 sample indices, in no particular order; *n_outliers, zeroed
 * by the caller, counts them; past outlier_cap entries err bit 4 (16) is set)
 * for nsvf_field_exact_dev. */
int nsvf_field_samples_bf16_dev(int64_t capacity, const int64_t *n_samples_dev,
                                const int32_t *voxel, const float *xyz_dist, int64_t n_voxels,
                                int64_t n_keys, float voxel_size, const float *centers,
                                const int32_t *feats, const float *values,
                                const void *const weights[5], const float *const biases[5],
                                float *out, int64_t *outliers, int64_t *n_outliers,
                                int64_t outlier_cap, int32_t *err, void *stream);

/* flag_outliers: the outlier list of nsvf_field_samples_bf16_dev for a field
 * evaluated elsewhere: samples s < min(*n_samples_dev, capacity)
 * (n_samples_dev may be NULL: capacity samples) with a trilinear coordinate
 * outside [-0.5, 1.5] in voxel[s] (computed as nsvf_trilinear_embed does)
 * are appended to list (*n_list zeroed by the caller; err bit 4 past
 * list_cap). No reference counterpart. */
int nsvf_flag_outliers(int64_t capacity, const int64_t *n_samples_dev, const int32_t *voxel,
                       const float *xyz_dist, int64_t n_voxels, float voxel_size,
                       const float *centers, int64_t *list, int64_t *n_list, int64_t list_cap,
                       int32_t *err, void *stream);

/* field_exact_dev: the workloads' field (32 -> 4 x 128 -> 4, ReLU) at the
 * listed samples, in double-float arithmetic (pairs of FP32 numbers:
 * error-free TwoSum / TwoProduct transformations and the compensated Dot2
 * dot product), written over out[s] = (sigma, r, g, b), rounded once to FP32.
 * No reference counterpart: the reference evaluates these samples in FP32,
 * where their extrapolated trilinear weights (up to 1e5 and more) turn the
 * field's relative rounding error into colour errors far above 2e-3.
 * Samples are the served layout: ray row i < min(*n_rows_dev, rows_cap) owns
 * samples [offset[i], offset[i + 1]); its ray is ray_index[i] (NULL:
 * identity) with origin ray_start[ray * ray_start_stride] (stride 3, or 0 for
 * one shared origin) and direction ray_dir[ray * 3]; sample s sits at depth[s]
 * in voxel[s]. The position o + d t, the trilinear weights, the embedding and
 * every layer are computed in double-float. weights_t[l] = W_l transposed,
 * [in, out] FP32 (32x128, 128x128 x3, 128x4); biases FP32. The list is read
 * on the device: min(*n_list, list_cap) entries. out 16-byte aligned.
 * If n_refine_rows is not NULL, the row of every listed sample whose
 * re-evaluated |r|, |g| or |b| exceeds refine_above is appended to
 * refine_rows (*n_refine_rows zeroed by the caller; err bit 4 past
 * refine_cap) for nsvf_field_refine_fp32_dev. */
int nsvf_field_exact_dev(int64_t rows_cap, const int64_t *n_rows_dev, const int64_t *offset,
                         const int64_t *ray_index, const float *ray_start,
                         int64_t ray_start_stride, const float *ray_dir, const float *depth,
                         const int32_t *voxel, int64_t n_voxels, int64_t n_keys,
                         float voxel_size, const float *centers, const int32_t *feats,
                         const float *values, const float *const weights_t[5],
                         const float *const biases[5], const int64_t *list,
                         const int64_t *n_list, int64_t list_cap, float *out,
                         float refine_above, int64_t *refine_rows, int64_t *n_refine_rows,
                         int64_t refine_cap, int32_t *err, void *stream);

/* field_refine_fp32_dev: the rows (rays) listed by nsvf_field_exact_dev --
 * those whose far-outside sample has a colour magnitude above refine_above --
 * get every other sample's (sigma, r, g, b) evaluated again in FP32 on the
 * CUDA cores (interpolation as nsvf_trilinear_embed, the layers with FP32
 * weights and activations), written over out. Such a sample's colour C
 * multiplies the error of the transmittance in front of it; in BF16 that
 * error is about 1e-6 (800x800 c4 frame), so rays with C above ~1000 would
 * leave more than 1e-3 of colour error. Samples far outside their voxel keep
 * their double-float values. rows / *n_rows_list (capacity rows_list_cap)
 * index ray rows < min(*n_rays_dev, rays_cap) of the served layout
 * (offset [rows + 1]); samples past sample_cap are not touched. No reference
 * counterpart. */
int nsvf_field_refine_fp32_dev(const int64_t *rows, const int64_t *n_rows_list,
                               int64_t rows_list_cap, int64_t rays_cap,
                               const int64_t *n_rays_dev, const int64_t *offset,
                               int64_t sample_cap, const int32_t *voxel, const float *xyz_dist,
                               int64_t n_voxels, int64_t n_keys, float voxel_size,
                               const float *centers, const int32_t *feats, const float *values,
                               const float *const weights_t[5], const float *const biases[5],
                               float *out, void *stream);

/* ------------------------------------------------------------------------ */
/* Field MLP on the tensor cores                                             */

/* mlp_forward_bf16: the workloads' field MLP 32 -> 128 -> 128 -> 128 -> 128
 * -> 4 (ReLU between layers) with tcgen05 BF16 MMAs and FP32 accumulation;
 * replaces the nn.Linear stack the reference's field runs in FP32
 * (fairnr/modules/implicit.py:42-75). emb [n, 32] FP32 (rounded to bf16 on
 * load), weights[l] row-major [out, in] bf16 (128x32, 128x128 x3, 4x128),
 * biases[l] FP32, out [n, 4] = (sigma, r, g, b) FP32. Hidden activations are
 * rounded to bf16 between layers. Pointers 16-byte aligned. err bit 3: a
 * pipeline wait timed out (kernel stopped early). */
int nsvf_mlp_forward_bf16(int64_t n_samples, const float *emb, const void *const weights[5],
                          const float *const biases[5], float *out, int32_t *err, void *stream);

/* field_samples_bf16: trilinear interpolation (as nsvf_trilinear_embed,
 * bit-identical FP32 embedding) fused into the input stage of the
 * tensor-core MLP: voxel [n] int32, xyz_dist [n, 4] FP32 (x, y, z, .),
 * centers [n_voxels, 3], feats [n_voxels, 8] int32, values [n_keys, 32]
 * FP32 -> out [n, 4] = (sigma, r, g, b). The embedding never reaches HBM.
 * feats, values, xyz_dist, out 16-byte aligned. */
int nsvf_field_samples_bf16(int64_t n_samples, const int32_t *voxel, const float *xyz_dist,
                            int64_t n_voxels, int64_t n_keys, float voxel_size,
                            const float *centers, const int32_t *feats, const float *values,
                            const void *const weights[5], const float *const biases[5],
                            float *out, int32_t *err, void *stream);

/* field_samples_fp8: nsvf_field_samples_bf16 with the three 128x128 hidden
 * layers in FP8 E4M3 (tcgen05 kind::f8f6f4, FP32 accumulation), the precision
 * option for the field; the input layer and the (sigma, rgb) head stay BF16.
 * weights[0], weights[4]: bf16 as above; weights[1..3]: E4M3 bytes of
 * W_l * w_scale[l], row-major [128, 128], 16-byte aligned. scales (host) =
 * {w_scale[1..3], a_scale[1..3]}, all positive and finite: the activation
 * entering layer l is multiplied by a_scale[l] and rounded to E4M3
 * (saturating at +-448), and layer l's accumulators are multiplied by
 * 1 / (a_scale[l] * w_scale[l]) before its bias. No reference counterpart
 * (the reference's field is FP32). */
int nsvf_field_samples_fp8(int64_t n_samples, const int32_t *voxel, const float *xyz_dist,
                           int64_t n_voxels, int64_t n_keys, float voxel_size,
                           const float *centers, const int32_t *feats, const float *values,
                           const void *const weights[5], const float *const biases[5],
                           const float scales[6], float *out, int32_t *err, void *stream);

/* field_samples_fp8_dev: nsvf_field_samples_fp8 on *n_samples_dev samples
 * (at most `capacity`), one persistent CTA per SM; outlier list as
 * nsvf_field_samples_bf16_dev. */
int nsvf_field_samples_fp8_dev(int64_t capacity, const int64_t *n_samples_dev,
                               const int32_t *voxel, const float *xyz_dist, int64_t n_voxels,
                               int64_t n_keys, float voxel_size, const float *centers,
                               const int32_t *feats, const float *values,
                               const void *const weights[5], const float *const biases[5],
                               const float scales[6], float *out, int64_t *outliers,
                               int64_t *n_outliers, int64_t outlier_cap, int32_t *err,
                               void *stream);

/* wait_timeout_selftest: the failure path of the kernels' bounded waits,
 * without a fault. One CTA waits on an mbarrier phase that never completes;
 * after limit_ns (1 ns .. 1 s) the wait gives up, bit 3 (8) of *err is set
 * (the bit the tensor-core kernels set on a timed-out wait) and the kernel
 * returns, leaving the context usable. No reference counterpart (the
 * reference's kernels have no waits). */
int nsvf_wait_timeout_selftest(uint64_t limit_ns, int32_t *err, void *stream);

/* prune_scores_bf16: self-pruning scores (SparseVoxelEncoder.get_scores,
 * fairnr/modules/encoder.py:620-654) in one kernel: for every voxel v,
 * bits^3 points at the offset_points positions around centers[v]
 * (fairnr/data/geometry.py:229-238), their embedding, the MLP's sigma, and
 *   rule 0 (reference pruning, encoder.py:610): score[v] = min exp(-relu s)
 *   rule 1 (sigma * step rule):                score[v] = max 1 - exp(-relu(s) step)
 * reduced into score[v] (FP32 bits, as uint32) with atomics: initialise
 * score to 0x7f800000 (+inf) for rule 0 and 0 for rule 1. keep is then
 * 1 - score > th (rule 0) or score >= th (rule 1). */
int nsvf_prune_scores_bf16(int64_t n_voxels, int bits, int rule, float step, int64_t n_keys,
                           float voxel_size, const float *centers, const int32_t *feats,
                           const float *values, const void *const weights[5],
                           const float *const biases[5], uint32_t *score, int32_t *err,
                           void *stream);

/* prune_screen_bf16 + prune_exact_dev: the pruning mask of
 * SparseVoxelEncoder.pruning (fairnr/modules/encoder.py:605-618, get_scores
 * :620-654), decided exactly. With T = -ln(1 - th) (rule 0, the reference's
 * rule: keep = 1 - min exp(-relu sigma) > th, i.e. max sigma > T) or
 * T = -ln(1 - th) / step (rule 1: keep = max 1 - exp(-relu(sigma) step) >=
 * th, i.e. max sigma >= T), 0 < th < 1:
 *  - prune_screen_bf16 runs the tensor-core pass of nsvf_prune_scores_bf16
 *    (score as there) and also computes, per point, M = sum_j |W4[0][j]| h_j
 *    from its BF16 activations h. A point with sigma - band * M above T sets
 *    keep[v] = 1 (uint8, zeroed by the caller); a point with sigma + band * M
 *    >= T that did not is appended (row v * bits^3 + i, int64) to list
 *    (*n_list zeroed by the caller; past list_cap err bit 4 (16) is set: call
 *    again with a larger list). The BF16 error of sigma measured on the
 *    workloads' fields stays below 0.005 M; band = 0.02 leaves a factor 4.
 *  - prune_exact_dev evaluates the listed points of voxels not yet kept in
 *    double-float arithmetic (as nsvf_field_exact_dev; point positions with
 *    offset_points' FP32 operations, fairnr/data/geometry.py:229-238) and sets
 *    keep[v] = 1 when sigma reaches T (T passed as a double, compared as a
 *    double-float). weights_t / biases as nsvf_field_exact_dev.
 * The mask is that of the reference's rule evaluated without rounding error;
 * an FP32 evaluation agrees with it except for voxels whose max sigma lies
 * within FP32 rounding of T. */
int nsvf_prune_screen_bf16(int64_t n_voxels, int bits, int rule, float step, float threshold,
                           float band, int64_t n_keys, float voxel_size, const float *centers,
                           const int32_t *feats, const float *values,
                           const void *const weights[5], const float *const biases[5],
                           uint32_t *score, uint8_t *keep, int64_t *list, int64_t *n_list,
                           int64_t list_cap, int32_t *err, void *stream);
int nsvf_prune_exact_dev(int64_t n_voxels, int bits, int rule, double threshold, int64_t n_keys,
                         float voxel_size, const float *centers, const int32_t *feats,
                         const float *values, const float *const weights_t[5],
                         const float *const biases[5], const int64_t *list,
                         const int64_t *n_list, int64_t list_cap, uint8_t *keep, int32_t *err,
                         void *stream);

#ifdef __cplusplus
}
#endif
#endif /* NSVF_GB300_H */
