"""The c2 workload (seeded synthetic scene, embeddings, field weights and
cameras) for the CPU legs, built without the product package.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py): bench.py's reference arm
and CPU baseline time the oracle on this data, so that no product code (and
no product library) runs on those legs. tests/test_oracle_workload.py checks
that every array equals the product's own workload bit for bit.

* voxel centres on the reference grid (bbox2voxels,
  fairnr/modules/encoder.py:1053-1059) inside the shell |SDF| < 2 voxels of
  sphere(r=0.6) U torus(R=0.7, r=0.2 about z);
* the sparse-voxel octree from the oracle's EasyOctree restatement
  (build_easy_octree, fairnr/data/geometry.py:320-327);
* the encoder's corner table (fairnr/modules/encoder.py:266-271) and its
  precomputed centres, shifted by voxel/10 in x (encoder.py:381-383);
* N(0, 0.01^2) corner embeddings and the Xavier-uniform 4x128 field, from
  torch generators with the workload's seeds;
* 100 seeded cameras on the radius-4 sphere, 800x800 pinhole frames.
"""
import math

import numpy as np

from . import cpu


def grid(voxel_size, lo=-1.0, hi=1.0):
    """Reference grid centres in its enumeration order (numpy meshgrid 'xy':
    y slowest, then x, then z), float32 [n, 3]."""
    n = int(round((hi - lo) / voxel_size)) + 1
    ax = np.arange(n)
    gx, gy, gz = np.meshgrid(ax, ax, ax)
    cols = [g.reshape(-1).astype(np.float32) * np.float64(voxel_size) + lo for g in (gx, gy, gz)]
    return np.stack(cols).T.astype(np.float32)


def shell_points(voxel_size):
    c = grid(voxel_size)
    p = c.astype(np.float64)
    sphere = np.linalg.norm(p, axis=-1) - 0.6
    ring = np.sqrt(p[:, 0] ** 2 + p[:, 1] ** 2) - 0.7
    torus = np.sqrt(ring ** 2 + p[:, 2] ** 2) - 0.2
    return c[np.abs(np.minimum(sphere, torus)) < 2.0 * voxel_size]


def octree(points, half_voxel):
    """(node centres [Nn, 3] float32, children [Nn, 9] int32)."""
    coords, residual = cpu.discretize_points(points, half_voxel)
    span = int((coords.max(0) - coords.min(0)).max())
    depth = int(np.ceil(np.log2(np.float32(span)))) - 1
    center = ((coords.max(0) + coords.min(0)) / 2).astype(np.float32)
    cen, chi = cpu.build_octree(center, coords, depth)
    return (cen.astype(np.float32) * np.float32(half_voxel) + residual).astype(np.float32), chi


def corner_table(points, voxel_size):
    """(sorted unique integer corner keys [Kc, 3], feats [V, 8] int64)."""
    coords, _ = cpu.discretize_points(points, voxel_size * 0.5)
    keys0 = (coords[:, None, :] + cpu.corner_offsets().astype(np.int64)[None]).reshape(-1, 3)
    keys, inv = np.unique(keys0, axis=0, return_inverse=True)
    return keys, inv.reshape(-1, 8).astype(np.int64)


def embeddings(num_keys, dim=32, std=0.01, seed=1):
    import torch
    g = torch.Generator().manual_seed(seed)
    return (torch.randn(num_keys, dim, generator=g) * std).numpy()


def field_weights(seed=2, dims=(32, 128, 128, 128, 128, 4)):
    """[(W [out, in], b [out]) float32] of the Xavier-uniform ReLU MLP with
    zero biases, drawn in layer order from one seeded generator."""
    import torch
    g = torch.Generator().manual_seed(seed)
    out = []
    for a, b in zip(dims[:-1], dims[1:]):
        bound = math.sqrt(6.0 / (a + b))
        W = (torch.rand(b, a, generator=g) * 2 - 1) * bound
        out.append((W.numpy(), np.zeros(b, np.float32)))
    return out


def camera(index, n=100, radius=4.0, seed=0):
    v = np.random.RandomState(seed).normal(size=(n, 3))
    return (radius * v / np.linalg.norm(v, axis=1, keepdims=True))[index]


def frame(index, size=800):
    """(ray_start [3] float32, ray_dir [size*size, 3] float32) of camera
    `index % 100`, looking at the origin, focal 80/64 of the width, rays
    through pixel centres in row-major order."""
    cam = camera(index % 100)
    f = -cam / np.linalg.norm(cam)
    up = np.array([0.0, 0.0, 1.0])
    if abs(np.dot(up, f)) > 0.99:
        up = np.array([0.0, 1.0, 0.0])
    r = np.cross(f, up)
    r /= np.linalg.norm(r)
    d = np.cross(f, r)
    rot = np.stack([r, d, f], 1)
    focal = 80.0 * size / 64.0
    j, i = np.meshgrid(np.arange(size) + 0.5, np.arange(size) + 0.5)
    dc = np.stack([(j - size / 2.0) / focal, (i - size / 2.0) / focal, np.ones_like(i)],
                  -1).reshape(-1, 3)
    dw = dc @ rot.T
    dw /= np.linalg.norm(dw, axis=1, keepdims=True)
    return cam.astype(np.float32), dw.astype(np.float32)


def c2_scene(voxel_size=1.0 / 64):
    """Everything the CPU render needs for the c2 (or, at 1/128, c4) scene."""
    p = shell_points(voxel_size)
    cen, chi = octree(p, voxel_size / 2)
    _, feats = corner_table(p, voxel_size)
    values = embeddings(int(feats.max()) + 1)
    shifted = p.copy()
    shifted[:, 0] += np.float32(voxel_size / 10)
    return dict(voxel_size=voxel_size, points=p, octree=(cen, chi), feats=feats, values=values,
                centers_shifted=shifted, weights_np=field_weights())
