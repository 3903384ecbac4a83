"""Front end of the CPU oracle.

TEST INFRASTRUCTURE ONLY (see oracle/__init__.py). Two layers:

1. ctypes wrappers of the C restatement in oracle/clib_oracle.c, taking and
   returning numpy arrays with the reference op layouts
   (fairnr/clib/src/intersect.cpp, fairnr/clib/src/sample.cpp,
   fairnr/clib/src/octree.cpp).
2. numpy restatements of the torch-level parts of the path:
   the op wrappers' batching (fairnr/clib/__init__.py), the encoder's
   intersection post-processing and sampling glue
   (fairnr/modules/encoder.py:498-556, fairnr/models/nsvf.py:65-75),
   trilinear interpolation (fairnr/data/geometry.py:195-200 with the corner
   order of offset_points, fairnr/data/geometry.py:229-238), the BASELINE
   stand-in field MLP, and compositing (fairnr/modules/renderer.py:77-232).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(HERE, "_build")
_SO = os.path.join(_BUILD, "liboracle.so")
_SRC = os.path.join(HERE, "clib_oracle.c")
MAX_DEPTH = 10000.0

_lib = None


def build():
    """Compile clib_oracle.c (plain C, no contraction) into oracle/_build/."""
    os.makedirs(_BUILD, exist_ok=True)
    if os.path.exists(_SO) and os.path.getmtime(_SO) >= os.path.getmtime(_SRC):
        return _SO
    tmp = _SO + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O2", "-std=c99", "-ffp-contract=off", "-fPIC", "-shared",
                           _SRC, "-o", tmp, "-lm"])
    os.replace(tmp, _SO)
    return _SO


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        i, f, i64 = ctypes.c_int, ctypes.c_float, ctypes.c_int64
        _lib.or_aabb_intersect.argtypes = [i, i, i, f, i, P, P, P, P, P, P]
        _lib.or_svo_intersect.argtypes = [i, i, i, f, i, P, P, P, P, P, P, P]
        _lib.or_svo_intersect.restype = i
        _lib.or_ball_intersect.argtypes = [i, i, i, f, i, P, P, P, P, P, P]
        _lib.or_triangle_intersect.argtypes = [i, i, i, f, f, i, P, P, P, P, P, P]
        _lib.or_uniform_sampling.argtypes = [i, i, i, i, f, P, P, P, P, P, P, P]
        _lib.or_inverse_cdf.argtypes = [i, i, i, i, f, P, P, P, P, P, P, P, P, P, P, P]
        _lib.or_build_octree.argtypes = [P, P, i64, i, P, P, i64]
        _lib.or_build_octree.restype = i64
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


# --------------------------------------------------------------------------
# layer 1: the _ext ops (fairnr/clib/src/binding.cpp:11-20)

def aabb_intersect(ray_start, ray_dir, points, voxelsize, n_max):
    rs, rd, pts = _c(ray_start, np.float32), _c(ray_dir, np.float32), _c(points, np.float32)
    b, m = rs.shape[:2]
    n = pts.shape[1]
    idx = np.empty((b, m, n_max), np.int32)
    lo = np.empty((b, m, n_max), np.float32)
    hi = np.empty((b, m, n_max), np.float32)
    lib().or_aabb_intersect(b, n, m, voxelsize, n_max, _p(rs), _p(rd), _p(pts), _p(idx), _p(lo), _p(hi))
    return idx, lo, hi


def svo_intersect(ray_start, ray_dir, points, children, voxelsize, n_max):
    rs, rd, pts = _c(ray_start, np.float32), _c(ray_dir, np.float32), _c(points, np.float32)
    ch = _c(children, np.int32)
    b, m = rs.shape[:2]
    n = pts.shape[1]
    idx = np.empty((b, m, n_max), np.int32)
    lo = np.empty((b, m, n_max), np.float32)
    hi = np.empty((b, m, n_max), np.float32)
    ov = lib().or_svo_intersect(b, n, m, voxelsize, n_max, _p(rs), _p(rd), _p(pts), _p(ch),
                                _p(idx), _p(lo), _p(hi))
    if ov:
        raise RuntimeError("oracle: octree traversal stack overflow on %d rays" % ov)
    return idx, lo, hi


def ball_intersect(ray_start, ray_dir, points, radius, n_max):
    rs, rd, pts = _c(ray_start, np.float32), _c(ray_dir, np.float32), _c(points, np.float32)
    b, m = rs.shape[:2]
    n = pts.shape[1]
    idx = np.empty((b, m, n_max), np.int32)
    lo = np.empty((b, m, n_max), np.float32)
    hi = np.empty((b, m, n_max), np.float32)
    lib().or_ball_intersect(b, n, m, radius, n_max, _p(rs), _p(rd), _p(pts), _p(idx), _p(lo), _p(hi))
    return idx, lo, hi


def triangle_intersect(ray_start, ray_dir, faces, cagesize, blur, n_max):
    """faces [b, n, 9] -> idx [b, m, n_max], depth [b, m, 3 n_max], uv [b, m, 2 n_max]."""
    rs, rd, F = _c(ray_start, np.float32), _c(ray_dir, np.float32), _c(faces, np.float32)
    b, m = rs.shape[:2]
    n = F.shape[1]
    idx = np.empty((b, m, n_max), np.int32)
    depth = np.empty((b, m, 3 * n_max), np.float32)
    uv = np.empty((b, m, 2 * n_max), np.float32)
    lib().or_triangle_intersect(b, n, m, float(cagesize), float(blur), n_max, _p(rs), _p(rd),
                                _p(F), _p(idx), _p(depth), _p(uv))
    return idx, depth, uv


def uniform_ray_sampling(pts_idx, min_depth, max_depth, noise, step_size, max_steps):
    I, lo, hi = _c(pts_idx, np.int32), _c(min_depth, np.float32), _c(max_depth, np.float32)
    U = _c(noise, np.float32)
    b, m, H = I.shape
    assert U.shape == (b, m, max_steps)
    si = np.empty((b, m, max_steps), np.int32)
    sd = np.empty((b, m, max_steps), np.float32)
    ss = np.empty((b, m, max_steps), np.float32)
    lib().or_uniform_sampling(b, m, H, max_steps, step_size, _p(I), _p(lo), _p(hi), _p(U),
                              _p(si), _p(sd), _p(ss))
    return si, sd, ss


def inverse_cdf_sampling(pts_idx, min_depth, max_depth, noise, probs, steps, fixed_step_size,
                         tail_row=None, next_row=None):
    I, lo, hi = _c(pts_idx, np.int32), _c(min_depth, np.float32), _c(max_depth, np.float32)
    U, pr, st = _c(noise, np.float32), _c(probs, np.float32), _c(steps, np.float32)
    b, m, H = I.shape
    M = U.shape[-1]
    tr = _c(tail_row, np.int64) if tail_row is not None else None
    nr = _c(next_row, np.int64) if next_row is not None else None
    si = np.empty((b, m, M), np.int32)
    sd = np.empty((b, m, M), np.float32)
    ss = np.empty((b, m, M), np.float32)
    lib().or_inverse_cdf(b, m, H, M, fixed_step_size, _p(I), _p(lo), _p(hi), _p(U), _p(pr), _p(st),
                         _p(tr), _p(nr), _p(si), _p(sd), _p(ss))
    return si, sd, ss


def build_octree(center, points, depth):
    """The _ext.build_octree op: integer points [V,3] -> (centers [Nn,3] int32, children [Nn,9] int32)."""
    c = _c(center, np.float32).reshape(3)
    pts = _c(points, np.int64)
    V = pts.shape[0]
    cap = max(16, V * 3 + 64)
    while True:
        cen = np.empty((cap, 3), np.int32)
        chi = np.empty((cap, 9), np.int32)
        n = lib().or_build_octree(_p(c), _p(pts), V, int(depth), _p(cen), _p(chi), cap)
        if n == -2:
            cap *= 2
            continue
        if n < 0:
            raise RuntimeError("oracle: octree build failed (%d)" % n)
        return cen[:n].copy(), chi[:n].copy()


# --------------------------------------------------------------------------
# layer 2: op wrappers and module glue

def discretize_points(points, voxel_size):
    """fairnr/data/geometry.py:241-247, in float32 like the reference tensors."""
    points = points.astype(np.float32)
    mn = points.min(0, keepdims=True)
    q = (points - mn) / np.float32(voxel_size)
    idx = np.round(q).astype(np.int64)   # torch.round_ = round half to even, like np.round
    # the mean accumulated in float64 (a float32 running sum over 500k
    # voxels drifts by 1e-2; torch's float32 mean is accurate here)
    residual = (points - idx.astype(np.float32) * np.float32(voxel_size)).mean(0, keepdims=True,
                                                                                  dtype=np.float64)
    return idx, residual.astype(np.float32)


def inverse_cdf_rows(N, G=200, chunk=800):
    """Row maps of the reference op wrapper's layout (fairnr/clib/__init__.py:234-270):
    rays padded to G*K (padding rows copy ray 0), viewed as [G, K], launched in
    column chunks of `chunk`. Returns (tail_row, next_row) for rays 0..N-1."""
    K = -(-N // G)
    orig = np.arange(G * K).reshape(G, K)
    orig = np.where(orig < N, orig, 0)
    tail = np.zeros(G * K, np.int64)
    nxt = np.zeros(G * K, np.int64)
    for c0 in range(0, K, chunk):
        W = min(chunk, K - c0)
        sub = orig[:, c0:c0 + W].reshape(-1)        # launch rows in memory order
        pos = (np.arange(G)[:, None] * K + c0 + np.arange(W)[None, :]).reshape(-1)
        f = np.arange(G * W)
        tail[pos] = sub[(f // W) * W]
        nx = np.full(G * W, -1, np.int64)
        nx[:-1] = sub[1:]
        nxt[pos] = nx
    return tail[:N], nxt[:N]


def inverse_cdf_op(pts_idx, min_depth, max_depth, probs, steps, noise_rows, fixed_step_size=-1.0):
    """The InverseCDFRaySampling op (fairnr/clib/__init__.py:231-300) for [N,H]
    inputs; `noise_rows` is the wrapper's noise viewed as [G*K, M] (only rows
    0..N-1 are read). Returns outputs truncated to the longest valid row."""
    N, H = pts_idx.shape
    tail, nxt = inverse_cdf_rows(N)
    M = noise_rows.shape[-1]
    si, sd, ss = inverse_cdf_sampling(pts_idx[None], min_depth[None], max_depth[None],
                                      noise_rows[None, :N], probs[None], steps[None],
                                      fixed_step_size, tail, nxt)
    si, sd, ss = si[0], sd[0], ss[0]
    L = int((si != -1).sum(-1).max()) if N else 0
    return si[:, :L], sd[:, :L], ss[:, :L]


def parallel_ray_sampling(march, pts_idx, min_depth, max_depth, noise=None):
    """The back-up parallel uniform sampler (fairnr/clib/__init__.py:303-349)
    on one chunk of [R, H] sorted hit lists, in float32 numpy. noise [R, K]
    is the clamped jitter (None: 0.5). The depth sort is stable in the
    concatenation order exits, entries, steps (the reference's torch.sort
    leaves ties unspecified; at a face shared by two voxels this puts the
    exit first, so the next segment takes the entered voxel's id). Returns
    (idx, depth, dists) truncated to the largest kept count."""
    f32 = np.float32
    pts_idx = np.asarray(pts_idx)
    lo = np.asarray(min_depth, f32)
    hi = np.asarray(max_depth, f32)
    R, H = pts_idx.shape
    first = lo.min(1)
    last = np.where(hi == f32(MAX_DEPTH), f32(0), hi).max(1).astype(f32)
    K = int(f32(f32((last - first).max()) / f32(march))) if R else 0
    k = np.arange(K, dtype=f32)[None, :]
    jit = f32(0.5) if noise is None else np.asarray(noise, f32)[:, :K]
    delta = ((k + jit).astype(f32) * f32(march)).astype(f32)
    u = (lo[:, :1] + delta).astype(f32)
    cnt = (u[:, :, None] >= lo[:, None, :]).sum(-1) - 1
    uid = np.take_along_axis(pts_idx, cnt, 1)
    d = np.concatenate([hi, lo, u], 1)
    ids = np.concatenate([pts_idx, pts_idx, uid], 1)
    order = np.argsort(d, axis=1, kind="stable")
    d = np.take_along_axis(d, order, 1)
    ids = np.take_along_axis(ids, order, 1)
    dist = (d[:, 1:] - d[:, :-1]).astype(f32)
    mid = (f32(0.5) * (d[:, 1:] + d[:, :-1]).astype(f32)).astype(f32)
    min_ids = (mid[:, :, None] >= lo[:, None, :]).sum(-1) - 1
    max_ids = (mid[:, :, None] >= hi[:, None, :]).sum(-1)
    bad = (max_ids != min_ids) | (mid > last[:, None]) | (dist == 0)
    mid = np.where(bad, f32(MAX_DEPTH), mid)
    order = np.argsort(mid, axis=1, kind="stable")
    mid = np.take_along_axis(mid, order, 1)
    dist = np.where(bad, f32(0), dist)
    dist = np.take_along_axis(dist, order, 1)
    ids = np.take_along_axis(np.where(bad, -1, ids[:, :-1]), order, 1)
    n = int((~np.take_along_axis(bad, order, 1)).sum(-1).max()) if R else 0
    return ids[:, :n], mid[:, :n], dist[:, :n]


def shared_face_ids_agree(idx, ref_idx, depth, dists, pts_idx, min_depth, max_depth):
    """Checker for parallel_ray_sampling outputs against the reference's:
    ids equal everywhere except segments that start at a face shared by two
    consecutive hit voxels (one's exit equals the next one's entry), where
    the reference's torch.sort picks either voxel; there the two ids must be
    those two voxels. Returns the number of such segments."""
    n = 0
    for r, c in zip(*np.nonzero(idx != ref_idx)):
        left = np.float64(depth[r, c]) - np.float64(dists[r, c]) / 2
        ok = False
        for j in range(pts_idx.shape[1] - 1):
            if pts_idx[r, j + 1] == -1:
                break
            if max_depth[r, j] == min_depth[r, j + 1] and abs(left - max_depth[r, j]) <= 1e-5 and \
                    {int(idx[r, c]), int(ref_idx[r, c])} == {int(pts_idx[r, j]), int(pts_idx[r, j + 1])}:
                ok = True
                break
        if not ok:
            raise AssertionError("segment %d of row %d: id %d vs %d away from a shared face"
                                 % (c, r, idx[r, c], ref_idx[r, c]))
        n += 1
    return n


def prepare_hierarchical(depth, dists, voxel_idx, probs, fixed_fine_num_samples=0,
                         fine_num_sample_ratio=0):
    """Hierarchical resampling's fine-pass inputs (fairnr/models/nerf.py:
    64-79, fairnr/models/nsvf.py:83-87) in float32: intervals [t - d/2,
    t + d/2], the coarse probs plus 1e-5 normalised per ray (sequential
    slot-order sum), steps = fixed_fine_num_samples or the coarse count times
    fine_num_sample_ratio."""
    f32 = np.float32
    depth, dists = np.asarray(depth, f32), np.asarray(dists, f32)
    lo = (depth - dists * f32(0.5)).astype(f32)
    hi = (depth + dists * f32(0.5)).astype(f32)
    safe = (np.asarray(probs, f32) + f32(1e-5)).astype(f32)
    tot = np.add.accumulate(safe, axis=-1, dtype=f32)[..., -1:]
    pr = (safe / tot).astype(f32)
    steps = np.ones(safe.shape[:-1], f32)
    if fixed_fine_num_samples > 0:
        steps = (steps * f32(fixed_fine_num_samples)).astype(f32)
    if fine_num_sample_ratio > 0:
        steps = ((voxel_idx != -1).sum(-1).astype(f32) * f32(fine_num_sample_ratio)).astype(f32)
    return lo, hi, np.asarray(voxel_idx), pr, steps


def sort_hits(idx, lo, hi):
    """Encoder post-processing (fairnr/modules/encoder.py:518-523): misses to
    MAX_DEPTH, stable sort by min_depth, gather."""
    lo = np.where(idx == -1, np.float32(MAX_DEPTH), lo).astype(np.float32)
    hi = np.where(idx == -1, np.float32(MAX_DEPTH), hi).astype(np.float32)
    order = np.argsort(lo, axis=-1, kind="stable")
    return (np.take_along_axis(idx, order, -1), np.take_along_axis(lo, order, -1),
            np.take_along_axis(hi, order, -1))


def probs_steps(idx, lo, hi, step_size):
    """fairnr/models/nsvf.py:65-74 in float32, the per-ray sum taken one slot
    at a time in slot order (np.add.accumulate is a sequential loop)."""
    d = np.where(idx == -1, np.float32(0), (hi - lo).astype(np.float32)).astype(np.float32)
    if d.shape[-1] == 0:
        tot = np.zeros(d.shape[:-1] + (1,), np.float32)
    else:
        tot = np.add.accumulate(d, axis=-1, dtype=np.float32)[..., -1:]
    with np.errstate(invalid="ignore", divide="ignore"):
        probs = (d / tot).astype(np.float32)
    steps = (tot[..., 0] / np.float32(step_size)).astype(np.float32)
    return probs, steps


def corner_offsets():
    """The 8 corner offsets in offset_points order (meshgrid of (x,y,z), 'ij')."""
    c = np.array([-1.0, 1.0])
    ox, oy, oz = np.meshgrid(c, c, c, indexing="ij")
    return np.stack([ox.reshape(-1), oy.reshape(-1), oz.reshape(-1)], 1)


def trilinear_embed(xyz, voxel_idx, centers, feats, values, voxel_size):
    """SparseVoxelEncoder.forward embedding (fairnr/modules/encoder.py:578-590)
    in float64: p = (x - c)/vs + .5, q = corners/2 + .5,
    w_k = prod(p*q + (1-p)*(1-q)), emb = sum_k w_k * values[feats[v, k]]."""
    xyz = np.asarray(xyz, np.float64)
    c = np.asarray(centers, np.float64)[voxel_idx]
    p = (xyz - c) / float(voxel_size) + 0.5
    q = corner_offsets() * 0.5 + 0.5
    w = (p[:, None, :] * q[None] + (1 - p[:, None, :]) * (1 - q[None])).prod(-1)   # [Ns, 8]
    v = np.asarray(values, np.float64)[np.asarray(feats)[voxel_idx]]                # [Ns, 8, E]
    return (w[..., None] * v).sum(1)


def mlp_forward(emb, weights):
    """Stand-in field MLP: ReLU hidden layers, linear head; out[:,0] = sigma,
    out[:,1:4] = rgb. weights = [(W [out,in], b [out]), ...] like nn.Linear."""
    x = np.asarray(emb, np.float64)
    for li, (W, b) in enumerate(weights):
        x = x @ np.asarray(W, np.float64).T + np.asarray(b, np.float64)
        if li < len(weights) - 1:
            x = np.maximum(x, 0)
    return x[:, 0], x[:, 1:4]


def composite(sigma, rgb, depth, dist, mask, sigma_scale=7.0):
    """VolumeRenderer compositing (fairnr/modules/renderer.py:117-121, 193-218)
    in float64 over [R, M] samples (mask = valid samples):
    fe = relu(sigma)*dist*7, a = 1-exp(-fe), T = exp(-cumsum(shifted fe)),
    p = a*T, depth = sum p*t, missed = 1-sum p, color = sum p*rgb."""
    fe = np.where(mask, np.maximum(sigma, 0) * dist * sigma_scale, 0.0)
    sh = np.concatenate([np.zeros_like(fe[:, :1]), fe[:, :-1]], 1)
    a = 1 - np.exp(-fe)
    T = np.exp(-np.cumsum(sh, 1))
    p = a * T
    return {
        "probs": p,
        "depths": (depth * p).sum(-1),
        "missed": 1 - p.sum(-1),
        "colors": (np.where(mask[..., None], rgb, 0.0) * p[..., None]).sum(1),
    }
