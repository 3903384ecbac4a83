"""Drop-in for the reference's native module ``fairnr.clib._ext``.

Same function names, argument order, dtypes and output shapes as the
pybind11 module of fairnr/clib/src/binding.cpp:11-20; each call launches the
sm_103a kernels of libnsvf_gb300.so on the current CUDA stream. Precondition
failures raise RuntimeError like the reference's TORCH_CHECKs
(fairnr/clib/include/utils.h:10-30); a failed launch raises NsvfError instead
of exiting the process.

Kernel-detected input problems (a malformed octree, a noise tensor too short
for the requested steps) are OR-ed into a per-device error word rather than
trapping; ``check_errors()`` synchronises and raises if any was recorded.
The sampling wrappers of nsvf_gb300.clib, which synchronise anyway for their
output width, check it on every call.
"""
import contextlib
import ctypes

import numpy as np
import torch

from ._lib import LIB, check

NSVF_ERR_OCTREE = -3
NSVF_ERR_CAPACITY = -4

_err_words = {}

# Optional per-op CUDA-event timing on the launching stream (used by bench.py
# to report per-kernel durations inside its timed region).
KERNEL_TIMING = False
kernel_events = []


@contextlib.contextmanager
def _timed(name, device):
    if not KERNEL_TIMING:
        yield
        return
    s = torch.cuda.Event(enable_timing=True)
    e = torch.cuda.Event(enable_timing=True)
    s.record(torch.cuda.current_stream(device))
    yield
    e.record(torch.cuda.current_stream(device))
    kernel_events.append((name, s, e))


def kernel_times_ms():
    """{op: {"launches", "total_ms", "avg_ms"}} of the recorded events (synchronises)."""
    torch.cuda.synchronize()
    out = {}
    for name, s, e in kernel_events:
        d = out.setdefault(name, {"launches": 0, "total_ms": 0.0})
        d["launches"] += 1
        d["total_ms"] += s.elapsed_time(e)
    for d in out.values():
        d["avg_ms"] = d["total_ms"] / d["launches"]
        d["total_ms"] = round(d["total_ms"], 4)
        d["avg_ms"] = round(d["avg_ms"], 4)
    return out


def _stream(t):
    return ctypes_stream(t.device)


def ctypes_stream(device):
    return torch.cuda.current_stream(device).cuda_stream


def error_word(device):
    """Per-device int32 error word the kernels OR their findings into."""
    key = torch.device(device).index if torch.device(device).index is not None \
        else torch.cuda.current_device()
    w = _err_words.get(key)
    if w is None:
        w = torch.zeros(1, dtype=torch.int32, device=torch.device("cuda", key))
        _err_words[key] = w
    return w


def check_errors(device=None):
    """Raise if any kernel on `device` recorded an input error since the last check."""
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else device
    w = error_word(dev)
    v = int(w.item())
    if v:
        w.zero_()
        what = []
        if v & 1:
            what.append("malformed octree (child id out of range, cycle or too deep)")
        if v & 2:
            what.append("a ray needed more sample slots than max_steps / noise columns")
        if v & 4:
            what.append("a voxel or corner id out of range in trilinear interpolation")
        if v & 8:
            what.append("a tensor-core pipeline wait timed out")
        if v & 16:
            what.append("more samples far outside their voxel than the outlier list holds")
        raise RuntimeError("nsvf_gb300: " + "; ".join(what))


def _ptr(t):
    return t.data_ptr() if t is not None else None


def _need(cond, msg):
    if not cond:
        raise RuntimeError(msg)


def _check_cuda_contig(name, t):
    _need(t.is_cuda, "%s must be a CUDA tensor" % name)
    _need(t.is_contiguous(), "%s must be a contiguous tensor" % name)


def _check_float(name, t):
    _check_cuda_contig(name, t)
    _need(t.dtype == torch.float32, "%s must be a float tensor" % name)


def _check_int(name, t):
    _check_cuda_contig(name, t)
    _need(t.dtype == torch.int32, "%s must be an int tensor" % name)


def _batch_pts(points, b):
    bp = points.size(0)
    _need(bp == b or bp == 1, "points batch (%d) must be 1 or match the ray batch (%d)" % (bp, b))
    return bp


def aabb_intersect(ray_start, ray_dir, points, voxelsize, n_max):
    """fairnr/clib/src/intersect.cpp:49-75: -> (idx int32, min_depth, max_depth) [B, M, n_max]."""
    for n, t in (("ray_start", ray_start), ("ray_dir", ray_dir), ("points", points)):
        _check_float(n, t)
    B, M = ray_start.shape[:2]
    bp = _batch_pts(points, B)
    N = points.size(1)
    dev = ray_start.device
    idx = torch.empty(B, M, n_max, dtype=torch.int32, device=dev)
    lo = torch.empty(B, M, n_max, dtype=torch.float32, device=dev)
    hi = torch.empty(B, M, n_max, dtype=torch.float32, device=dev)
    check(LIB.nsvf_aabb_intersect(B, bp, N, M, float(voxelsize), int(n_max), _ptr(ray_start),
                                  _ptr(ray_dir), _ptr(points), _ptr(idx), _ptr(lo), _ptr(hi),
                                  _stream(ray_start)), "aabb_intersect")
    return idx, lo, hi


def _svo_workspace(bp, n, dev):
    nbytes = int(LIB.nsvf_svo_workspace_bytes(bp, n))
    return torch.empty(max(nbytes, 16), dtype=torch.uint8, device=dev)


def svo_intersect(ray_start, ray_dir, points, children, voxelsize, n_max):
    """fairnr/clib/src/intersect.cpp:84-112: -> (idx, min_depth, max_depth) [B, M, n_max]."""
    for n, t in (("ray_start", ray_start), ("ray_dir", ray_dir), ("points", points)):
        _check_float(n, t)
    _check_int("children", children)
    B, M = ray_start.shape[:2]
    bp = _batch_pts(points, B)
    N = points.size(1)
    _need(children.shape[:2] == points.shape[:2] and children.size(2) == 9,
          "children must be [B, N, 9] matching points")
    dev = ray_start.device
    idx = torch.empty(B, M, n_max, dtype=torch.int32, device=dev)
    lo = torch.empty(B, M, n_max, dtype=torch.float32, device=dev)
    hi = torch.empty(B, M, n_max, dtype=torch.float32, device=dev)
    ws = _svo_workspace(bp, N, dev)
    check(LIB.nsvf_svo_intersect(B, bp, N, M, float(voxelsize), int(n_max), _ptr(ray_start),
                                 _ptr(ray_dir), _ptr(points), _ptr(children), _ptr(idx), _ptr(lo),
                                 _ptr(hi), _ptr(error_word(dev)), _ptr(ws), _stream(ray_start)),
          "svo_intersect")
    return idx, lo, hi


def svo_intersect_sorted(ray_start, ray_dir, points, children, voxelsize, n_max):
    """svo_intersect plus the encoder's post-processing (fairnr/modules/encoder.py:518-524):
    -> (idx, min_depth, max_depth) sorted by min_depth with misses at 10000, hits [B, M] bool."""
    for n, t in (("ray_start", ray_start), ("ray_dir", ray_dir), ("points", points)):
        _check_float(n, t)
    _check_int("children", children)
    _need(n_max <= 128, "sorted SVO intersection supports n_max <= 128")
    B, M = ray_start.shape[:2]
    bp = _batch_pts(points, B)
    N = points.size(1)
    dev = ray_start.device
    idx = torch.empty(B, M, n_max, dtype=torch.int32, device=dev)
    lo = torch.empty(B, M, n_max, dtype=torch.float32, device=dev)
    hi = torch.empty(B, M, n_max, dtype=torch.float32, device=dev)
    hits = torch.empty(B, M, dtype=torch.uint8, device=dev)
    ws = _svo_workspace(bp, N, dev)
    with _timed("svo_intersect_sorted", dev):
        check(LIB.nsvf_svo_intersect_sorted(B, bp, N, M, float(voxelsize), int(n_max),
                                            _ptr(ray_start), _ptr(ray_dir), _ptr(points),
                                            _ptr(children), _ptr(idx), _ptr(lo), _ptr(hi),
                                            _ptr(hits), _ptr(error_word(dev)), _ptr(ws),
                                            _stream(ray_start)), "svo_intersect_sorted")
    return idx, lo, hi, hits.bool()


class SvoGrid:
    """Leaf-grid form of ONE octree on its device, for nsvf_svo_intersect_grid:
    the blob of nsvf_svo_grid_build (built on the host from a copy of the
    octree) and the packed octree of nsvf_svo_pack, both kept for the
    octree's lifetime. `ok` is False when the tree is not in leaf-grid form;
    callers then use the depth-first kernel (svo_intersect_sorted)."""

    def __init__(self, centers, children, voxel_size):
        _check_float("centers", centers)
        _check_int("children", children)
        _need(centers.dim() == 2 and centers.size(1) == 3 and children.dim() == 2 and
              children.size(1) == 9 and children.size(0) == centers.size(0),
              "one octree: centers [N, 3], children [N, 9]")
        dev = centers.device
        self.n = int(centers.size(0))
        self.voxel_size = float(voxel_size)
        self.centers = centers.contiguous()
        self.children = children.contiguous()
        c = self.centers.detach().cpu().numpy()
        ch = self.children.detach().cpu().numpy()
        nbytes = ctypes.c_int64(0)
        st = LIB.nsvf_svo_grid_build(self.n, self.voxel_size, c.ctypes.data, ch.ctypes.data, None,
                                     0, ctypes.byref(nbytes))
        self.ok = st == NSVF_ERR_CAPACITY
        if not self.ok:
            if st != NSVF_ERR_OCTREE:
                check(st, "svo_grid_build")
            return
        blob = np.zeros(int(nbytes.value), np.uint8)
        check(LIB.nsvf_svo_grid_build(self.n, self.voxel_size, c.ctypes.data, ch.ctypes.data,
                                      blob.ctypes.data, blob.size, None), "svo_grid_build")
        info = np.zeros(6, np.int32)
        check(LIB.nsvf_svo_grid_info(blob.ctypes.data, info.ctypes.data), "svo_grid_info")
        self.info = info                     # host int32[6], passed to every call
        self.lines = tuple(int(v) for v in info[:3])
        self.n_leaves, self.n_flagged = int(info[3]), int(info[4])
        self.grid = torch.from_numpy(blob).to(dev)
        self.packed = _svo_workspace(1, self.n, dev)
        check(LIB.nsvf_svo_pack(self.n, self.voxel_size, _ptr(self.centers), _ptr(self.children),
                                _ptr(self.packed), _stream(self.centers)), "svo_pack")
        self._lists = {}

    def bytes(self):
        return self.grid.numel() + self.packed.numel() if self.ok else 0

    def list_workspace(self, rays, dev):
        """The ray-list scratch for calls of `rays` rays on the current stream
        (kept per stream: calls on one stream run in order)."""
        key = _stream(self.grid)
        ws = self._lists.get(key)
        need = int(LIB.nsvf_svo_grid_list_bytes(rays))
        if ws is None or ws.numel() < need:
            ws = torch.empty(need, dtype=torch.uint8, device=dev)
            self._lists[key] = ws
        return ws

    def intersect_into(self, R, n_max, ro, rd, idx, lo, hi, hits, stream, list_ws=None,
                       err=None, padded=True):
        """nsvf_svo_intersect_grid on raw device pointers (R rays); `err` (a
        device int32 tensor) defaults to the device's error word. padded=False
        (nsvf_svo_intersect_grid_rows): a row ends at its first -1 and missed
        rays' rows are not written (for readers that stop there, such as
        nsvf_gather_probs)."""
        ws = list_ws if list_ws is not None else self.list_workspace(R, self.grid.device)
        if err is None:
            err = error_word(self.grid.device)
        check(LIB.nsvf_svo_intersect_grid_rows(
            R, self.n, self.voxel_size, int(n_max), ro, rd, _ptr(self.centers),
            _ptr(self.children), _ptr(self.grid), self.info.ctypes.data, _ptr(self.packed),
            _ptr(ws), idx, lo, hi, hits,
            _ptr(err), int(bool(padded)), stream), "svo_intersect_grid_rows")


def svo_intersect_grid(grid, ray_start, ray_dir, n_max):
    """Sorted SVO intersection through a SvoGrid: ray_start, ray_dir [R, 3]
    (or [1, R, 3]) -> the outputs of svo_intersect_sorted with B = 1."""
    _need(grid.ok, "the octree is not in leaf-grid form")
    _need(n_max <= 128, "sorted SVO intersection supports n_max <= 128")
    for n, t in (("ray_start", ray_start), ("ray_dir", ray_dir)):
        _check_float(n, t)
    rs = ray_start.reshape(-1, 3).contiguous()
    rd = ray_dir.reshape(-1, 3).contiguous()
    _need(rs.shape == rd.shape, "one origin per ray")
    R = rd.size(0)
    dev = rd.device
    idx = torch.empty(1, R, n_max, dtype=torch.int32, device=dev)
    lo = torch.empty(1, R, n_max, dtype=torch.float32, device=dev)
    hi = torch.empty(1, R, n_max, dtype=torch.float32, device=dev)
    hits = torch.empty(1, R, dtype=torch.uint8, device=dev)
    with _timed("svo_intersect_grid", dev):
        grid.intersect_into(R, n_max, _ptr(rs), _ptr(rd), _ptr(idx), _ptr(lo), _ptr(hi),
                            _ptr(hits), _stream(rd))
    return idx, lo, hi, hits.bool()


def ball_intersect(ray_start, ray_dir, points, radius, n_max):
    """fairnr/clib/src/intersect.cpp:15-41: -> (idx, min_depth, max_depth) [B, M, n_max]."""
    for n, t in (("ray_start", ray_start), ("ray_dir", ray_dir), ("points", points)):
        _check_float(n, t)
    B, M = ray_start.shape[:2]
    bp = _batch_pts(points, B)
    N = points.size(1)
    dev = ray_start.device
    idx = torch.empty(B, M, n_max, dtype=torch.int32, device=dev)
    lo = torch.empty(B, M, n_max, dtype=torch.float32, device=dev)
    hi = torch.empty(B, M, n_max, dtype=torch.float32, device=dev)
    check(LIB.nsvf_ball_intersect(B, bp, N, M, float(radius), int(n_max), _ptr(ray_start),
                                  _ptr(ray_dir), _ptr(points), _ptr(idx), _ptr(lo), _ptr(hi),
                                  _stream(ray_start)), "ball_intersect")
    return idx, lo, hi


def triangle_intersect(ray_start, ray_dir, face_points, cagesize, blur, n_max):
    """fairnr/clib/src/intersect.cpp:120-145: face_points [B or 1, F, 9] ->
    (idx [B, M, n_max], depth [B, M, 3 n_max], uv [B, M, 2 n_max])."""
    for n, t in (("ray_start", ray_start), ("ray_dir", ray_dir), ("face_points", face_points)):
        _check_float(n, t)
    B, M = ray_start.shape[:2]
    bf = _batch_pts(face_points, B)
    N = face_points.size(1)
    dev = ray_start.device
    idx = torch.empty(B, M, n_max, dtype=torch.int32, device=dev)
    depth = torch.empty(B, M, 3 * n_max, dtype=torch.float32, device=dev)
    uv = torch.empty(B, M, 2 * n_max, dtype=torch.float32, device=dev)
    check(LIB.nsvf_triangle_intersect(B, bf, N, M, float(cagesize), float(blur), int(n_max),
                                      _ptr(ray_start), _ptr(ray_dir), _ptr(face_points),
                                      _ptr(idx), _ptr(depth), _ptr(uv), _stream(ray_start)),
          "triangle_intersect")
    return idx, depth, uv


def uniform_ray_sampling(pts_idx, min_depth, max_depth, uniform_noise, step_size, max_steps):
    """fairnr/clib/src/sample.cpp:23-55: -> (sampled_idx, sampled_depth, sampled_dists) [B, M, max_steps]."""
    _check_int("pts_idx", pts_idx)
    for n, t in (("min_depth", min_depth), ("max_depth", max_depth),
                 ("uniform_noise", uniform_noise)):
        _check_float(n, t)
    B, M, H = pts_idx.shape
    _need(uniform_noise.shape[:2] == (B, M) and uniform_noise.size(2) >= max_steps,
          "uniform_noise must be [B, M, >= max_steps]")
    if uniform_noise.size(2) != max_steps:
        uniform_noise = uniform_noise[..., :max_steps].contiguous()
    dev = pts_idx.device
    si = torch.empty(B, M, max_steps, dtype=torch.int32, device=dev)
    sd = torch.empty(B, M, max_steps, dtype=torch.float32, device=dev)
    ss = torch.empty(B, M, max_steps, dtype=torch.float32, device=dev)
    check(LIB.nsvf_uniform_ray_sampling(B, M, H, int(max_steps), float(step_size), _ptr(pts_idx),
                                        _ptr(min_depth), _ptr(max_depth), _ptr(uniform_noise),
                                        _ptr(si), _ptr(sd), _ptr(ss), _ptr(error_word(dev)),
                                        _stream(pts_idx)), "uniform_ray_sampling")
    return si, sd, ss


def inverse_cdf_sampling_rows(pts_idx, min_depth, max_depth, noise, probs, steps,
                              fixed_step_size, layout, max_steps, max_len=None):
    """Inverse-CDF sampling over [rows, H] inputs with an explicit launch layout
    (see nsvf_inverse_cdf_sampling in include/nsvf_gb300.h). noise is
    [>= rows, >= max_steps] or None for the deterministic 0.5 jitter."""
    rows, H = pts_idx.shape
    dev = pts_idx.device
    si = torch.empty(rows, max_steps, dtype=torch.int32, device=dev)
    sd = torch.empty(rows, max_steps, dtype=torch.float32, device=dev)
    ss = torch.empty(rows, max_steps, dtype=torch.float32, device=dev)
    lay = (torch.tensor(layout, dtype=torch.int64)).contiguous()
    with _timed("inverse_cdf_sampling", dev):
        check(LIB.nsvf_inverse_cdf_sampling(
            rows, H, int(max_steps), noise.size(-1) if noise is not None else 0,
            float(fixed_step_size), _ptr(pts_idx), _ptr(min_depth), _ptr(max_depth), _ptr(noise),
            _ptr(probs), _ptr(steps), lay.data_ptr(), _ptr(si), _ptr(sd), _ptr(ss), _ptr(max_len),
            _ptr(error_word(dev)), _stream(pts_idx)), "inverse_cdf_sampling")
    return si, sd, ss


def inverse_cdf_sampling(pts_idx, min_depth, max_depth, uniform_noise, probs, steps,
                         fixed_step_size):
    """fairnr/clib/src/sample.cpp:58-96 over [B, M, H] inputs (max_steps = noise.size(-1)):
    -> (sampled_idx, sampled_depth, sampled_dists) [B, M, max_steps]."""
    _check_int("pts_idx", pts_idx)
    for n, t in (("min_depth", min_depth), ("max_depth", max_depth),
                 ("uniform_noise", uniform_noise), ("probs", probs), ("steps", steps)):
        _check_float(n, t)
    B, M, H = pts_idx.shape
    S = uniform_noise.size(-1)
    rows = B * M
    si, sd, ss = inverse_cdf_sampling_rows(
        pts_idx.view(rows, H), min_depth.view(rows, H), max_depth.view(rows, H),
        uniform_noise.view(rows, S), probs.view(rows, H), steps.view(rows), fixed_step_size,
        (max(M, 1), max(M, 1), rows, max(B, 1)), S)
    return si.view(B, M, S), sd.view(B, M, S), ss.view(B, M, S)


def parallel_ray_sampling_rows(pts_idx, min_depth, max_depth, noise, march_size, n_steps,
                               sampled_idx, sampled_depth, sampled_dists, count):
    """nsvf_parallel_ray_sampling over [rows, H] hit lists with n_steps
    uniform steps per ray (noise [rows, n_steps] or None for 0.5), into
    [rows, W] outputs and the kept counts [rows] (int32)."""
    rows, H = pts_idx.shape
    W = sampled_idx.shape[1] if sampled_idx.dim() == 2 else 0
    dev = pts_idx.device
    with _timed("parallel_ray_sampling", dev):
        check(LIB.nsvf_parallel_ray_sampling(rows, H, int(n_steps), float(march_size),
                                             _ptr(pts_idx), _ptr(min_depth), _ptr(max_depth),
                                             _ptr(noise), W, _ptr(sampled_idx),
                                             _ptr(sampled_depth), _ptr(sampled_dists),
                                             _ptr(count), ctypes_stream(dev)),
              "parallel_ray_sampling")


def ray_probs(pts_idx, min_depth, max_depth, step_size):
    """The sampling distribution of NSVFModel.intersecting
    (fairnr/models/nsvf.py:65-74) on the GPU: [..., H] sorted hit lists ->
    (probs [..., H], steps [...]). Each ray's segment lengths are summed in
    slot order (nsvf_ray_probs); the served chain uses the same order."""
    H = pts_idx.size(-1)
    idx = pts_idx.reshape(-1, H)
    if idx.dtype != torch.int32:
        idx = idx.int()
    idx = idx.contiguous()
    lo = min_depth.reshape(-1, H).float().contiguous()
    hi = max_depth.reshape(-1, H).float().contiguous()
    rows = idx.shape[0]
    dev = idx.device
    probs = torch.empty(rows, H, dtype=torch.float32, device=dev)
    steps = torch.empty(rows, dtype=torch.float32, device=dev)
    with _timed("ray_probs", dev):
        check(LIB.nsvf_ray_probs(rows, H, float(step_size), _ptr(idx), _ptr(lo), _ptr(hi),
                                 _ptr(probs), _ptr(steps), ctypes_stream(dev)), "ray_probs")
    return probs.view(pts_idx.shape), steps.view(pts_idx.shape[:-1])


def build_octree(center, points, depth):
    """fairnr/clib/src/octree.cpp:125-136 (host build): center [3], points [V, 3]
    integer coordinates -> (centers [Nn, 3] int32, children [Nn, 9] int32) on points' device."""
    import ctypes
    import numpy as np
    c = np.ascontiguousarray(center.detach().float().cpu().numpy().reshape(3), dtype=np.float32)
    p = np.ascontiguousarray(points.detach().cpu().numpy().reshape(-1, 3), dtype=np.int64)
    cp = ctypes.c_void_p(c.ctypes.data)
    pp = ctypes.c_void_p(p.ctypes.data)
    n = LIB.nsvf_build_octree(cp, pp, p.shape[0], int(depth), None, None, 0)
    if n < 0:
        check(int(n), "build_octree")
    cen = np.empty((n, 3), np.int32)
    chi = np.empty((n, 9), np.int32)
    n2 = LIB.nsvf_build_octree(cp, pp, p.shape[0], int(depth), ctypes.c_void_p(cen.ctypes.data),
                               ctypes.c_void_p(chi.ctypes.data), n)
    if n2 < 0:
        check(int(n2), "build_octree")
    dev = points.device
    return torch.from_numpy(cen).to(dev), torch.from_numpy(chi).to(dev)


def camera_rays(intrinsics, inv_RT, H, W, h=None, w=None, first=0, n=None, device=None):
    """Rays of an H x W image read at h x w, in the reference's camera
    convention (ImageReader eval path: get_uv, get_ray_direction), on the
    GPU: intrinsics (fx, fy, cx, cy), inv_RT camera-to-world [3 or 4, 4].
    Returns ray_start [n, 3] and ray_dir [n, 3] for pixels first..first+n-1
    of the w-wide grid (all by default). Same kernel as nsvf_camera_rays."""
    h = H if h is None else h
    w = W if w is None else w
    n = h * w - first if n is None else n
    dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
    M = torch.as_tensor(inv_RT, dtype=torch.float32).reshape(-1, 4)[:3].reshape(-1)
    fx, fy, cx, cy = [float(x) for x in intrinsics]
    cam = torch.cat([torch.tensor([fx, fy, cx, cy]), M.cpu(),
                     torch.tensor([float(W / w), float(H / h), float(w), float(first)])]).to(dev)
    ro = torch.empty(n, 3, dtype=torch.float32, device=dev)
    rd = torch.empty(n, 3, dtype=torch.float32, device=dev)
    with _timed("camera_rays", dev):
        check(LIB.nsvf_camera_rays(n, cam.data_ptr(), ro.data_ptr(), rd.data_ptr(),
                                   ctypes_stream(dev)), "camera_rays")
    return ro, rd
