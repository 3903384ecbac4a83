/*
 * C entry points around the reference's CUDA kernels compiled for the CPU
 * (see oracle/build_ref.py). TEST INFRASTRUCTURE ONLY.
 *
 * Each entry point runs the reference kernel once per block with a single
 * "thread" (blockDim.x = 1), so every block's stride loop visits all of its
 * rays in order. Rays are independent in these kernels, so this is the same
 * computation the GPU does with many threads.
 */
#include "cuda_utils.h"

ref_cpu_idx threadIdx = {0, 0, 0}, blockIdx = {0, 0, 0}, blockDim = {1, 1, 1};

#include REF_INTERSECT_KERNELS
#include REF_SAMPLE_KERNELS

extern "C" {

void ref_aabb_intersect(int b, int n, int m, float voxelsize, int n_max,
                        const float *ray_start, const float *ray_dir, const float *points,
                        int *idx, float *min_depth, float *max_depth) {
  for (int g = 0; g < b; ++g) {
    blockIdx.x = g;
    aabb_intersect_point_kernel(b, n, m, voxelsize, n_max, ray_start, ray_dir, points,
                                idx, min_depth, max_depth);
  }
}

void ref_svo_intersect(int b, int n, int m, float voxelsize, int n_max,
                       const float *ray_start, const float *ray_dir, const float *points,
                       const int *children, int *idx, float *min_depth, float *max_depth) {
  for (int g = 0; g < b; ++g) {
    blockIdx.x = g;
    svo_intersect_point_kernel(b, n, m, voxelsize, n_max, ray_start, ray_dir, points,
                               children, idx, min_depth, max_depth);
  }
}

void ref_ball_intersect(int b, int n, int m, float radius, int n_max,
                        const float *ray_start, const float *ray_dir, const float *points,
                        int *idx, float *min_depth, float *max_depth) {
  for (int g = 0; g < b; ++g) {
    blockIdx.x = g;
    ball_intersect_point_kernel(b, n, m, radius, n_max, ray_start, ray_dir, points,
                                idx, min_depth, max_depth);
  }
}

void ref_triangle_intersect(int b, int n, int m, float cagesize, float blur, int n_max,
                            const float *ray_start, const float *ray_dir, const float *face_points,
                            int *idx, float *depth, float *uv) {
  for (int g = 0; g < b; ++g) {
    blockIdx.x = g;
    triangle_intersect_point_kernel(b, n, m, cagesize, blur, n_max, ray_start, ray_dir,
                                    face_points, idx, depth, uv);
  }
}

void ref_uniform_ray_sampling(int b, int num_rays, int max_hits, int max_steps, float step_size,
                              const int *pts_idx, const float *min_depth, const float *max_depth,
                              const float *uniform_noise, int *sampled_idx, float *sampled_depth,
                              float *sampled_dists) {
  for (int g = 0; g < b; ++g) {
    blockIdx.x = g;
    uniform_ray_sampling_kernel(b, num_rays, max_hits, max_steps, step_size, pts_idx, min_depth,
                                max_depth, uniform_noise, sampled_idx, sampled_depth, sampled_dists);
  }
}

void ref_inverse_cdf_sampling(int b, int num_rays, int max_hits, int max_steps,
                              float fixed_step_size, const int *pts_idx, const float *min_depth,
                              const float *max_depth, const float *uniform_noise,
                              const float *probs, const float *steps, int *sampled_idx,
                              float *sampled_depth, float *sampled_dists) {
  for (int g = 0; g < b; ++g) {
    blockIdx.x = g;
    inverse_cdf_sampling_kernel(b, num_rays, max_hits, max_steps, fixed_step_size, pts_idx,
                                min_depth, max_depth, uniform_noise, probs, steps, sampled_idx,
                                sampled_depth, sampled_dists);
  }
}

}  // extern "C"
