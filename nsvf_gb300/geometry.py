"""Geometry helpers of the hot path (drop-in for the parts of
fairnr/data/geometry.py the sparse-voxel encoder uses).

* discretize_points  fairnr/data/geometry.py:241-247
* offset_points      fairnr/data/geometry.py:229-238
* trilinear_interp   fairnr/data/geometry.py:195-200 (torch form, kept for API
                     compatibility; the encoder uses the fused CUDA kernel)
* build_easy_octree  fairnr/data/geometry.py:320-327 (octree built by the
                     native host builder, nsvf_build_octree)
* splitting_points   fairnr/data/geometry.py:250-274
* bbox2voxels        fairnr/modules/encoder.py:1053-1059
* ray, fill_in       fairnr/data/geometry.py:160-161, 303-317
"""
import numpy as np
import torch
import torch.nn.functional as F

from . import ext

INF = 1000.0


def ray(ray_start, ray_dir, depths):
    return ray_start + ray_dir * depths


def discretize_points(voxel_points, voxel_size):
    """Voxel centres/corners -> integer grid coordinates (rounded, relative to
    the minimum point) and the mean residual (fairnr/data/geometry.py:
    discretize_points). The residuals are the reference's FP32 values; their
    mean is taken in float64 and rounded once, so it is the same on every
    device: torch's FP32 mean is not (on CUDA it multiplies the sum by 1/N,
    one ulp off the exact mean of the c2 shell's identical residuals, and every
    octree centre, slab distance and sample would inherit that ulp)."""
    minimal = voxel_points.min(dim=0, keepdim=True)[0]
    coords = ((voxel_points - minimal) / voxel_size).round_().long()
    res = voxel_points - coords.type_as(voxel_points) * voxel_size
    residual = res.double().mean(0, keepdim=True).to(voxel_points.dtype)
    return coords, residual


def offset_points(point_xyz, quarter_voxel=1, offset_only=False, bits=2):
    """The bits^3 sub-cell offsets ((2i+1) - bits)/(bits-1) per axis in
    meshgrid (x, y, z) order, scaled by quarter_voxel and added to each point."""
    c = torch.arange(1, 2 * bits, 2, device=point_xyz.device)
    ox, oy, oz = torch.meshgrid([c, c, c], indexing="ij")
    offset = (torch.cat([ox.reshape(-1, 1), oy.reshape(-1, 1), oz.reshape(-1, 1)], 1)
              .type_as(point_xyz) - bits) / float(bits - 1)
    if not offset_only:
        return point_xyz.unsqueeze(1) + offset.unsqueeze(0).type_as(point_xyz) * quarter_voxel
    return offset.type_as(point_xyz) * quarter_voxel


def trilinear_interp(p, q, point_feats):
    weights = (p * q + (1 - p) * (1 - q)).prod(dim=-1, keepdim=True)
    if point_feats.dim() == 2:
        point_feats = point_feats.view(point_feats.size(0), 8, -1)
    return (weights * point_feats).sum(1)


def bbox2voxels(bbox, voxel_size):
    vox_min, vox_max = np.asarray(bbox[:3], np.float64), np.asarray(bbox[3:6], np.float64)
    steps = np.round((vox_max - vox_min) / voxel_size).astype(np.int64) + 1
    x, y, z = [c.reshape(-1).astype(np.float32) for c in
               np.meshgrid(np.arange(steps[0]), np.arange(steps[1]), np.arange(steps[2]))]
    x = x * np.float64(voxel_size) + vox_min[0]
    y = y * np.float64(voxel_size) + vox_min[1]
    z = z * np.float64(voxel_size) + vox_min[2]
    return np.stack([x, y, z]).T.astype(np.float32)


def build_easy_octree(points, half_voxel):
    """Flattened sparse-voxel octree of the voxel centres `points` [V, 3]:
    (centers [Nn, 3] float, children [Nn, 9] int32), leaves = rows 0..V-1,
    root = last row."""
    coords, residual = discretize_points(points, half_voxel)
    ranges = coords.max(0)[0] - coords.min(0)[0]
    depths = torch.log2(ranges.max().float()).ceil_().long() - 1
    center = (coords.max(0)[0] + coords.min(0)[0]) / 2
    centers, children = ext.build_octree(center, coords, int(depths))
    centers = centers.to(points.device).float() * half_voxel + residual
    return centers, children.to(points.device)


def splitting_points(point_xyz, point_feats, values, half_voxel):
    """Split every voxel into 8 and re-interpolate the corner embeddings
    (fairnr/data/geometry.py:250-274)."""
    quarter_voxel = half_voxel * .5
    new_points = offset_points(point_xyz, quarter_voxel).reshape(-1, 3)
    old_coords = discretize_points(point_xyz, quarter_voxel)[0]
    new_coords = offset_points(old_coords).reshape(-1, 3)
    new_keys0 = offset_points(new_coords).reshape(-1, 3)
    new_keys, new_feats = torch.unique(new_keys0, dim=0, sorted=True, return_inverse=True)
    new_keys_idx = new_feats.new_zeros(new_keys.size(0)).scatter_(
        0, new_feats, torch.arange(new_keys0.size(0), device=new_feats.device) // 64)
    new_feats = new_feats.reshape(-1, 8)
    if values is not None:
        p = (new_keys - old_coords[new_keys_idx]).type_as(point_xyz).unsqueeze(1) * .25 + 0.5
        q = offset_points(p, .5, offset_only=True).unsqueeze(0) + 0.5
        point_feats = point_feats[new_keys_idx]
        point_feats = F.embedding(point_feats, values).view(point_feats.size(0), -1)
        new_values = trilinear_interp(p, q, point_feats)
    else:
        new_values = None
    return new_points, new_feats, new_values, new_keys


def fill_in(shape, hits, input, initial=1.0):
    input_sizes = [k for k in input.size()]
    if (len(input_sizes) == len(shape)) and all(shape[i] == input_sizes[i] for i in range(len(shape))):
        return input
    if isinstance(initial, torch.Tensor):
        output = initial.expand(*shape)
    else:
        output = input.new_ones(*shape) * initial
    if len(shape) == 1:
        return output.masked_scatter(hits, input)
    return output.masked_scatter(hits.unsqueeze(-1).expand(*shape), input)


def voxel_corner_table(points, voxel_size):
    """The encoder's corner table (fairnr/modules/encoder.py:266-271): integer
    corner keys [Kc, 3] (sorted unique) and per-voxel corner ids feats [V, 8]."""
    coords, _ = discretize_points(points, voxel_size * .5)
    keys0 = offset_points(coords, 1.0).reshape(-1, 3)
    keys, feats = torch.unique(keys0, dim=0, sorted=True, return_inverse=True)
    return keys, feats.reshape(-1, 8)


def get_uv(H, W, h, w):
    """Pixel coordinates of an H x W image read at h x w: uv [2, h, w]
    float32 (u = column, v = row, integer positions scaled by W / w and
    H / h) and the ratios (fairnr/data/data_utils.py:57-65)."""
    v, u = np.mgrid[0:h, 0:w]
    uv = np.stack([u, v]).astype(np.float32)
    uv[0] = uv[0] * float(W / w)
    uv[1] = uv[1] * float(H / h)
    return uv, [float(H / h), float(W / w)]


def get_ray_direction(ray_start, uv, intrinsics, inv_RT, depths=None):
    """Unit ray directions [3, N] through pixels uv [2, N]: the point at
    `depths` (default 1) in camera space, (u - cx) / fx, (v - cy) / fy,
    mapped to the world by inv_RT [4, 4], minus ray_start [3], normalised
    with the reference's + 1e-8 (fairnr/data/geometry.py:116-122). intrinsics
    is a [4, 4] or [3, 3] matrix (fx, fy on the diagonal, cx, cy in the last
    column) or (fx, fy, cx, cy)."""
    z = 1 if depths is None else depths
    K = torch.as_tensor(intrinsics)
    if K.dim() == 2:
        fx, fy, cx, cy = K[0, 0], K[1, 1], K[0, 2], K[1, 2]
    else:
        fx, fy, cx, cy = K[0], K[1], K[2], K[3]
    x = (uv[0] - cx) / fx * z
    y = (uv[1] - cy) / fy * z
    cam = torch.stack([x, y, torch.ones_like(x) * z, torch.ones_like(x)])
    world = torch.matmul(inv_RT, cam)[:3]
    d = world - ray_start[:, None]
    return d / (d.norm(p=2, dim=0, keepdim=True) + 1e-8)
