"""ctypes front end of the reference's kernel bodies compiled for the CPU
(oracle/_ref/libref_clib.so, built by oracle/build_ref.py).

TEST INFRASTRUCTURE ONLY, and only where the reference checkout exists: it
pins the C oracle and generates tests/golden/. Same call shapes as the
layer-1 functions of oracle/cpu.py.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_ref", "libref_clib.so")
_lib = None


def available():
    return os.path.exists(SO)


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(SO)
        P = ctypes.c_void_p
        i, f = ctypes.c_int, ctypes.c_float
        _lib.ref_aabb_intersect.argtypes = [i, i, i, f, i, P, P, P, P, P, P]
        _lib.ref_svo_intersect.argtypes = [i, i, i, f, i, P, P, P, P, P, P, P]
        _lib.ref_ball_intersect.argtypes = [i, i, i, f, i, P, P, P, P, P, P]
        _lib.ref_triangle_intersect.argtypes = [i, i, i, f, f, i, P, P, P, P, P, P]
        _lib.ref_uniform_ray_sampling.argtypes = [i, i, i, i, f, P, P, P, P, P, P, P]
        _lib.ref_inverse_cdf_sampling.argtypes = [i, i, i, i, f, P, P, P, P, P, P, P, P, P]
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def _intersect(fn, ray_start, ray_dir, points, extra, size, n_max):
    rs, rd = _c(ray_start, np.float32), _c(ray_dir, np.float32)
    b, m = rs.shape[:2]
    n = points.shape[1]
    idx = np.zeros((b, m, n_max), np.int32)      # the reference allocates zeros
    lo = np.zeros((b, m, n_max), np.float32)
    hi = np.zeros((b, m, n_max), np.float32)
    args = [b, n, m, size, n_max, _p(rs), _p(rd), _p(points)]
    if extra is not None:
        args.append(_p(extra))
    fn(*args, _p(idx), _p(lo), _p(hi))
    return idx, lo, hi


def aabb_intersect(ray_start, ray_dir, points, voxelsize, n_max):
    return _intersect(lib().ref_aabb_intersect, ray_start, ray_dir, _c(points, np.float32), None,
                      voxelsize, n_max)


def svo_intersect(ray_start, ray_dir, points, children, voxelsize, n_max):
    return _intersect(lib().ref_svo_intersect, ray_start, ray_dir, _c(points, np.float32),
                      _c(children, np.int32), voxelsize, n_max)


def ball_intersect(ray_start, ray_dir, points, radius, n_max):
    return _intersect(lib().ref_ball_intersect, ray_start, ray_dir, _c(points, np.float32), None,
                      radius, n_max)


def uniform_ray_sampling(pts_idx, min_depth, max_depth, noise, step_size, max_steps):
    I, lo, hi = _c(pts_idx, np.int32), _c(min_depth, np.float32), _c(max_depth, np.float32)
    U = _c(noise, np.float32)
    b, m, H = I.shape
    si = np.full((b, m, max_steps), -1, np.int32)   # sample.cpp:39-47
    sd = np.zeros((b, m, max_steps), np.float32)
    ss = np.zeros((b, m, max_steps), np.float32)
    lib().ref_uniform_ray_sampling(b, m, H, max_steps, step_size, _p(I), _p(lo), _p(hi), _p(U),
                                   _p(si), _p(sd), _p(ss))
    return si, sd, ss


def inverse_cdf_sampling(pts_idx, min_depth, max_depth, noise, probs, steps, fixed_step_size):
    """One reference launch over [b, m, H]. The caller must give the arrays one
    spare row of pts_idx after the last ray if any ray can run its tail loop
    with curr_bin == max_hits (the reference reads one element past its row)."""
    I, lo, hi = _c(pts_idx, np.int32), _c(min_depth, np.float32), _c(max_depth, np.float32)
    U, pr, st = _c(noise, np.float32), _c(probs, np.float32), _c(steps, np.float32)
    b, m, H = I.shape
    M = U.shape[-1]
    # one spare -1 row so the past-the-end read of the last ray is defined
    Ipad = np.concatenate([I.reshape(-1), np.full(H, -1, np.int32)])
    si = np.full((b, m, M), -1, np.int32)
    sd = np.zeros((b, m, M), np.float32)
    ss = np.zeros((b, m, M), np.float32)
    lib().ref_inverse_cdf_sampling(b, m, H, M, fixed_step_size, _p(Ipad), _p(lo), _p(hi), _p(U),
                                   _p(pr), _p(st), _p(si), _p(sd), _p(ss))
    return si, sd, ss


def triangle_intersect(ray_start, ray_dir, faces, cagesize, blur, n_max):
    rs, rd, F = _c(ray_start, np.float32), _c(ray_dir, np.float32), _c(faces, np.float32)
    b, m = rs.shape[:2]
    n = F.shape[1]
    idx = np.zeros((b, m, n_max), np.int32)      # the reference allocates zeros
    depth = np.zeros((b, m, 3 * n_max), np.float32)
    uv = np.zeros((b, m, 2 * n_max), np.float32)
    lib().ref_triangle_intersect(b, n, m, float(cagesize), float(blur), n_max, _p(rs), _p(rd),
                                 _p(F), _p(idx), _p(depth), _p(uv))
    return idx, depth, uv
