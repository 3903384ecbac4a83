"""Seeded synthetic scenes and cameras for the benchmark workloads.

The reference trains on external datasets that are not available here; these
generators stand in for them with the voxel sizes, counts and camera set-ups
of the five workloads:

* c1 "small":  bbox [-1, 1]^3, voxel 0.25, centres within 0.8 of the origin
               (147 voxels on the reference's voxel grid), 64x64 view, f=80.
* c2 "shell":  voxel 1/64 on [-1, 1]^3, the shell |SDF| < 2 voxels of
               sphere(r=0.6) U torus(R=0.7, r=0.2 about z): 125,476 voxels,
               800x800 views from 100 seeded cameras on a radius-4 sphere.
* c4:          the same shell at voxel 1/128 (500,832 voxels).
* c5:          8 scenes of sphere/torus/box unions with 10k-400k voxels.

Voxel centres follow the reference's grid (bbox2voxels,
fairnr/modules/encoder.py:1053-1059): per axis round((max-min)/voxel)+1
centres, enumerated in numpy meshgrid 'xy' order (y slowest, then x, then z).
"""
import math

import numpy as np
import torch


def grid_centers(bbox_min, bbox_max, voxel_size):
    """Voxel centres of the reference grid, float32 [n, 3], in its order."""
    vmin = np.asarray(bbox_min, np.float64)
    vmax = np.asarray(bbox_max, np.float64)
    steps = np.round((vmax - vmin) / voxel_size).astype(np.int64) + 1
    x, y, z = [c.reshape(-1).astype(np.float32) for c in
               np.meshgrid(np.arange(steps[0]), np.arange(steps[1]), np.arange(steps[2]))]
    x = x * np.float64(voxel_size) + vmin[0]
    y = y * np.float64(voxel_size) + vmin[1]
    z = z * np.float64(voxel_size) + vmin[2]
    return np.stack([x, y, z]).T.astype(np.float32)


def sdf_sphere(p, r, c=(0.0, 0.0, 0.0)):
    return np.linalg.norm(p - np.asarray(c), axis=-1) - r


def sdf_torus(p, R, r, c=(0.0, 0.0, 0.0)):
    q = p - np.asarray(c)
    d = np.sqrt(q[:, 0] ** 2 + q[:, 1] ** 2) - R
    return np.sqrt(d ** 2 + q[:, 2] ** 2) - r


def sdf_box(p, half, c=(0.0, 0.0, 0.0)):
    q = np.abs(p - np.asarray(c)) - np.asarray(half)
    out = np.linalg.norm(np.maximum(q, 0.0), axis=-1)
    return out + np.minimum(np.max(q, axis=-1), 0.0)


def shell_voxels(voxel_size, sdf, width=2.0):
    """Centres of the voxels whose centre lies within `width` voxels of the
    zero set of `sdf` (float64 SDF of float32 centres)."""
    c = grid_centers([-1, -1, -1], [1, 1, 1], voxel_size)
    d = sdf(c.astype(np.float64))
    return c[np.abs(d) < width * voxel_size]


def scene_small():
    """c1: 147 voxels of size 0.25 inside the ball of radius 0.8."""
    c = grid_centers([-1, -1, -1], [1, 1, 1], 0.25)
    return c[np.linalg.norm(c.astype(np.float64), axis=-1) <= 0.8], 0.25


def sphere_torus_sdf(p):
    return np.minimum(sdf_sphere(p, 0.6), sdf_torus(p, 0.7, 0.2))


def scene_shell(voxel_size=1.0 / 64):
    """c2 (voxel 1/64) and c4 (voxel 1/128): sphere U torus shell."""
    return shell_voxels(voxel_size, sphere_torus_sdf), voxel_size


def serving_scenes(seed=5):
    """c5: eight sphere/torus/box unions at voxel sizes that put them between
    roughly 10k and 400k voxels."""
    rng = np.random.RandomState(seed)
    out = []
    sizes = [1 / 24, 1 / 32, 1 / 48, 1 / 64, 1 / 80, 1 / 96, 1 / 106, 1 / 116]
    for k, vs in enumerate(sizes):
        r = 0.35 + 0.25 * rng.rand()
        R, rt = 0.55 + 0.2 * rng.rand(), 0.1 + 0.1 * rng.rand()
        bh = 0.15 + 0.2 * rng.rand(3)
        bc = (rng.rand(3) - 0.5) * 0.6

        def sdf(p, r=r, R=R, rt=rt, bh=bh, bc=bc):
            return np.minimum(np.minimum(sdf_sphere(p, r), sdf_torus(p, R, rt)), sdf_box(p, bh, bc))

        out.append((shell_voxels(vs, sdf), vs))
    return out


# ---------------------------------------------------------------- cameras --

def sphere_cameras(n=100, radius=4.0, seed=0):
    """n seeded camera positions on the sphere of `radius` (float64 [n, 3])."""
    rng = np.random.RandomState(seed)
    v = rng.normal(size=(n, 3))
    return radius * v / np.linalg.norm(v, axis=1, keepdims=True)


def look_at(cam, target=(0.0, 0.0, 0.0)):
    """Camera-to-world rotation (columns = right, down, forward), OpenCV style."""
    f = np.asarray(target, np.float64) - cam
    f = f / np.linalg.norm(f)
    up = np.array([0.0, 0.0, 1.0])
    if abs(np.dot(up, f)) > 0.99:
        up = np.array([0.0, 1.0, 0.0])
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    d = np.cross(f, r)
    return np.stack([r, d, f], 1)


def pinhole_rays(cam, height, width, focal):
    """Rays through the pixel centres of a pinhole camera at `cam` looking at
    the origin: (ray_start [3] float32, ray_dir [H*W, 3] float32, unit length),
    pixels in row-major order."""
    R = look_at(np.asarray(cam, np.float64))
    j, i = np.meshgrid(np.arange(width) + 0.5, np.arange(height) + 0.5)
    d_cam = np.stack([(j - width / 2.0) / focal, (i - height / 2.0) / focal,
                      np.ones_like(i)], -1).reshape(-1, 3)
    d = d_cam @ R.T
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.asarray(cam, np.float32), d.astype(np.float32)


def small_view(seed=0):
    """c1 camera: distance 4, seeded direction, 64x64, focal 80 px."""
    cam = sphere_cameras(1, 4.0, seed)[0]
    return pinhole_rays(cam, 64, 64, 80.0)


def frame_view(index=0, size=800, seed=0):
    """c2/c4 camera `index` of the 100 seeded cameras; same field of view as
    c1 (focal = 80/64 of the width)."""
    cam = sphere_cameras(100, 4.0, seed)[index]
    return pinhole_rays(cam, size, size, 80.0 * size / 64.0)


# ------------------------------------------------------------- parameters --

def voxel_embeddings(num_keys, dim=32, std=0.01, seed=1, device="cpu"):
    g = torch.Generator().manual_seed(seed)
    return (torch.randn(num_keys, dim, generator=g) * std).to(device)


def stand_in_mlp_weights(in_dim=32, hidden=128, layers=4, out_dim=4, seed=2,
                         sigma_scale=1.0, sigma_bias=0.0):
    """Xavier-uniform weights and zero biases of the 4x128 ReLU field MLP
    (the reference's Linear init, fairnr/modules/module_utils.py:15-20):
    [(W [out, in], b [out]), ...], last layer -> (sigma, r, g, b).
    sigma_scale / sigma_bias rescale the density row of the last layer (test
    scenes use them to get an opaque, partly prunable field)."""
    g = torch.Generator().manual_seed(seed)
    dims = [in_dim] + [hidden] * layers + [out_dim]
    out = []
    for a, b in zip(dims[:-1], dims[1:]):
        bound = math.sqrt(6.0 / (a + b))
        W = (torch.rand(b, a, generator=g) * 2 - 1) * bound
        out.append((W, torch.zeros(b)))
    W, b = out[-1]
    W[0] *= sigma_scale
    b[0] = sigma_bias
    return out
