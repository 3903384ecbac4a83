"""Drop-in for the reference's op API ``fairnr.clib`` (fairnr/clib/__init__.py).

Same function names, arguments and outputs as the reference's
autograd.Function wrappers (all non-differentiable). What changes is how the
work reaches the GPU:

* Intersection: the reference splits the rays into up to 2048 groups and
  copies the voxel set / octree into every group to fill its one-block-per-
  row kernels (fairnr/clib/__init__.py:62-71, 101-111; ~8 GB of copies for the
  125k-voxel scene). Here one launch covers all rays against one copy.
* Sampling: the reference pads the rays to 200 (or 256) blocks and launches
  in slices of 800 columns (fairnr/clib/__init__.py:181-189, 234-270). Here
  one launch covers all rays; the two places where the reference's result
  depends on that blocking (see include/nsvf_gb300.h) are reproduced from the
  layout parameters, and the noise tensor is drawn with the same shape and
  torch RNG calls, so results are identical for the same seed.
"""
import numpy as np
import torch
from torch.autograd import Function

from . import ext

MAX_DEPTH = 10000.0


class BallRayIntersect(Function):
    @staticmethod
    def forward(ctx, radius, n_max, points, ray_start, ray_dir):
        inds, min_depth, max_depth = ext.ball_intersect(
            ray_start.float().contiguous(), ray_dir.float().contiguous(),
            points.float().contiguous(), radius, n_max)
        min_depth = min_depth.type_as(ray_start)
        max_depth = max_depth.type_as(ray_start)
        ctx.mark_non_differentiable(inds, min_depth, max_depth)
        return inds, min_depth, max_depth

    @staticmethod
    def backward(ctx, a, b, c):
        return None, None, None, None, None


ball_ray_intersect = BallRayIntersect.apply


class AABBRayIntersect(Function):
    @staticmethod
    def forward(ctx, voxelsize, n_max, points, ray_start, ray_dir):
        inds, min_depth, max_depth = ext.aabb_intersect(
            ray_start.float().contiguous(), ray_dir.float().contiguous(),
            points.float().contiguous(), float(voxelsize), int(n_max))
        min_depth = min_depth.type_as(ray_start)
        max_depth = max_depth.type_as(ray_start)
        ctx.mark_non_differentiable(inds, min_depth, max_depth)
        return inds, min_depth, max_depth

    @staticmethod
    def backward(ctx, a, b, c):
        return None, None, None, None, None


aabb_ray_intersect = AABBRayIntersect.apply


class SparseVoxelOctreeRayIntersect(Function):
    @staticmethod
    def forward(ctx, voxelsize, n_max, points, children, ray_start, ray_dir):
        inds, min_depth, max_depth = ext.svo_intersect(
            ray_start.float().contiguous(), ray_dir.float().contiguous(),
            points.float().contiguous(), children.int().contiguous(), float(voxelsize), int(n_max))
        min_depth = min_depth.type_as(ray_start)
        max_depth = max_depth.type_as(ray_start)
        ctx.mark_non_differentiable(inds, min_depth, max_depth)
        return inds, min_depth, max_depth

    @staticmethod
    def backward(ctx, a, b, c):
        return None, None, None, None, None, None


svo_ray_intersect = SparseVoxelOctreeRayIntersect.apply


class TriangleRayIntersect(Function):
    """fairnr/clib/__init__.py:136-173: rays against the mesh `faces` [F, 3]
    (vertex ids into `points`) -> inds [S, N, n_max], depth [S, N, n_max, 3]
    (t, min offset, max offset per hit), uv [S, N, 2 n_max]. The reference
    expands the face vertex table over up to 2048 ray groups; here one copy
    serves every row."""

    @staticmethod
    def forward(ctx, cagesize, blur_ratio, n_max, points, faces, ray_start, ray_dir):
        S, N = ray_start.shape[:2]
        face_points = torch.nn.functional.embedding(faces.reshape(-1, 3), points.reshape(-1, 3))
        face_points = face_points.reshape(1, -1, 9).float().contiguous()
        inds, depth, uv = ext.triangle_intersect(
            ray_start.float().contiguous(), ray_dir.float().contiguous(), face_points,
            float(cagesize), float(blur_ratio), int(n_max))
        depth = depth.type_as(ray_start).reshape(S, N, -1, 3)
        uv = uv.type_as(ray_start).reshape(S, N, -1)
        inds = inds.reshape(S, N, -1)
        ctx.mark_non_differentiable(inds, depth, uv)
        return inds, depth, uv

    @staticmethod
    def backward(ctx, a, b, c):
        return None, None, None, None, None, None, None


triangle_ray_intersect = TriangleRayIntersect.apply


def _truncate(sampled_idx, sampled_depth, sampled_dists, max_len):
    return sampled_idx[:, :max_len], sampled_depth[:, :max_len], sampled_dists[:, :max_len]


class UniformRaySampling(Function):
    @staticmethod
    def forward(ctx, pts_idx, min_depth, max_depth, step_size, max_ray_length, deterministic=False):
        G, N, P = 256, pts_idx.size(0), pts_idx.size(1)
        H = int(np.ceil(N / G)) * G
        max_steps = int(max_ray_length / step_size) + P * 2
        # noise drawn exactly as the reference: [G, H/G, max_steps], U(0, 1)
        noise = min_depth.new_zeros(H, max_steps)
        if deterministic:
            noise += 0.5
        else:
            noise = noise.uniform_()
        # the reference pads rows by repeating the FIRST H-N rows; rows are
        # independent except that a jitter of exactly 0 reads the previous
        # row's last id, which is the same element here
        si, sd, ss = ext.uniform_ray_sampling(
            pts_idx.int().contiguous().view(1, N, P), min_depth.float().contiguous().view(1, N, P),
            max_depth.float().contiguous().view(1, N, P),
            noise.float()[:N].contiguous().view(1, N, max_steps), float(step_size), max_steps)
        si, sd, ss = si.view(N, -1), sd.view(N, -1).type_as(min_depth), ss.view(N, -1).type_as(min_depth)
        ext.check_errors(pts_idx.device)
        max_len = si.ne(-1).sum(-1).max()
        si, sd, ss = _truncate(si, sd, ss, max_len)
        ctx.mark_non_differentiable(si, sd, ss)
        return si, sd, ss

    @staticmethod
    def backward(ctx, a, b, c):
        return None, None, None, None, None, None


uniform_ray_sampling = UniformRaySampling.apply


def inverse_cdf_layout(N, G=200, chunk=800):
    """The reference wrapper's launch layout for N rays: K = ceil(N/G) rays per
    block, launched `chunk` columns at a time (fairnr/clib/__init__.py:234-270)."""
    K = max(1, int(np.ceil(N / G)))
    return (K, chunk, N, G)


class InverseCDFRaySampling(Function):
    @staticmethod
    def forward(ctx, pts_idx, min_depth, max_depth, probs, steps, fixed_step_size=-1,
                deterministic=False):
        G, N, P = 200, pts_idx.size(0), pts_idx.size(1)
        H = int(np.ceil(N / G)) * G
        # max_steps over the padded rows (padding copies row 0): same as over N
        max_steps = int(steps.ceil().long().max()) + P
        if deterministic:
            noise = None   # the kernel's built-in 0.5 jitter
        else:
            # drawn exactly as the reference: [G, H/G, max_steps], clamped
            noise = min_depth.new_zeros(H, max_steps).uniform_().clamp(min=0.001, max=0.999)
            noise = noise.float()
        dev = pts_idx.device
        max_len = torch.zeros(1, dtype=torch.int32, device=dev)
        si, sd, ss = ext.inverse_cdf_sampling_rows(
            pts_idx.int().contiguous(), min_depth.float().contiguous(),
            max_depth.float().contiguous(), noise, probs.float().contiguous(),
            steps.float().contiguous(), float(fixed_step_size), inverse_cdf_layout(N),
            max_steps, max_len)
        sd, ss = sd.type_as(min_depth), ss.type_as(min_depth)
        ext.check_errors(dev)
        L = int(max_len.item())
        si, sd, ss = _truncate(si, sd, ss, L)
        ctx.mark_non_differentiable(si, sd, ss)
        return si, sd, ss

    @staticmethod
    def backward(ctx, a, b, c):
        return None, None, None, None, None, None, None


inverse_cdf_sampling = InverseCDFRaySampling.apply


@torch.no_grad()
def parallel_ray_sampling(MARCH_SIZE, pts_idx, min_depth, max_depth, deterministic=False):
    """The reference's back-up uniform sampler (fairnr/clib/__init__.py:
    303-383) on the GPU: nsvf_parallel_ray_sampling, a warp per ray. Same
    arguments and outputs (sampled_idx, sampled_depth, sampled_dists)
    [rays, width] with -1 / MAX_DEPTH / 0 padding.

    The reference works on chunks of 4096 rays; each chunk's number of
    uniform steps is int(longest ray / MARCH_SIZE) over that chunk (its
    rays' last exit minus first entry), its jitter a [rays, steps] uniform
    draw clamped to [0.01, 0.99] (0.5 with deterministic), and its output
    width the largest number of kept segments in the chunk; the chunks are
    then padded to the widest. All of that is kept, so a seeded call gives the
    reference's depths and distances. Ties between equal depths are ordered
    like a stable sort of [exits, entries, steps]: at a face shared by two
    voxels the segment after it takes the entered voxel's id (the reference's
    torch.sort leaves that order unspecified)."""
    chunk_size = 4096
    R, H = pts_idx.shape
    dev = pts_idx.device
    idx = pts_idx.int().contiguous()
    lo = min_depth.float().contiguous()
    hi = max_depth.float().contiguous()
    parts = []
    for i in range(0, max(R, 1), chunk_size):
        I, L, U = idx[i:i + chunk_size], lo[i:i + chunk_size], hi[i:i + chunk_size]
        n = I.shape[0]
        first = L.min(1)[0]
        last = U.masked_fill(U.eq(MAX_DEPTH), 0).max(1)[0]
        K = int((last - first).max() / MARCH_SIZE) if n else 0
        noise = None
        if not deterministic:
            noise = torch.empty(n, K, dtype=torch.float32, device=dev).uniform_() \
                .clamp(min=0.01, max=0.99).contiguous()
        W = max(2 * H + K - 1, 0)
        si = torch.empty(n, W, dtype=torch.int32, device=dev)
        sd = torch.empty(n, W, dtype=torch.float32, device=dev)
        ss = torch.empty(n, W, dtype=torch.float32, device=dev)
        cnt = torch.zeros(n, dtype=torch.int32, device=dev)
        ext.parallel_ray_sampling_rows(I, L, U, noise, float(MARCH_SIZE), K, si, sd, ss, cnt)
        w = int(cnt.max()) if n else 0
        parts.append((si[:, :w], sd[:, :w], ss[:, :w]))
    if len(parts) == 1:
        si, sd, ss = parts[0]
        return si.long() if pts_idx.dtype == torch.int64 else si, sd.type_as(min_depth), \
            ss.type_as(min_depth)
    width = max(p[0].shape[1] for p in parts)

    def pad(xs, value, dtype):
        out = torch.full((R, width), value, dtype=dtype, device=dev)
        st = 0
        for x in xs:
            out[st:st + x.shape[0], :x.shape[1]] = x
            st += x.shape[0]
        return out

    si = pad([p[0] for p in parts], -1, torch.int32)
    return si.long() if pts_idx.dtype == torch.int64 else si, \
        pad([p[1] for p in parts], MAX_DEPTH, torch.float32).type_as(min_depth), \
        pad([p[2] for p in parts], 0.0, torch.float32).type_as(min_depth)
