"""Served frame renderer: the hot path as a short chain of sm_103a kernels.

For one frame of rays of a resident scene:

1. nsvf_svo_intersect_sorted  -- octree traversal + depth sort (FP32, exact)
2. nsvf_compact_hits          -- order-preserving compaction of the hit rays
   (on a torch prefix sum of the hit flags)
3. nsvf_gather_probs          -- the hit rays' lists and their sampling
   distribution (fairnr/models/nsvf.py:65-74), warp per ray
4. nsvf_sample_count_dev / nsvf_sample_compact_dev -- the inverse-CDF walk
   (deterministic jitter, the reference's launch layout) writing only the
   valid samples, compacted per ray
5. nsvf_field_samples_bf16    -- corner-embedding interpolation fused into the
                                 tcgen05 BF16 field MLP (FP32 accumulation);
                                 embeddings and activations stay on chip
6. nsvf_composite_segments    -- compensated transmittance compositing into
                                 the frame (the background is filled first)

With the tensor-core field the whole chain runs on device-side counts (hit
rays, samples), so the host enqueues the frame while the traversal runs and
reads the counts once, at the end. The sample buffers keep a capacity across
frames; a frame that needs more is composited again with room for it.

Geometry (slab distances, sample depths and positions) is FP32 and comes from
the drop-in path's kernels. The one difference from the drop-in path is the
order of the per-ray sum of segment lengths in step 3 (a fixed warp order
instead of torch's reduction order); a ray whose sum rounds differently can
get samples shifted by that rounding. The MLP runs in BF16.
"""
import ctypes

import torch

from . import ext
from ._lib import LIB, check
from .functional import trilinear_embed
from .mlp import TensorCoreMLP


def _p(t):
    return t.data_ptr() if t is not None else None


class SceneState:
    """Device-resident scene: octree, shifted voxel centres, corner table,
    embeddings, field weights (FP32 and BF16), background."""

    def __init__(self, encoder, field, max_hits=None):
        states = encoder.precompute(id=None)
        self.voxel_size = float(encoder.voxel_size)
        self.step_size = float(encoder.step_size)
        self.max_hits = int(encoder.max_hits if max_hits is None else max_hits)
        self.octree_centers = states['voxel_octree_center_xyz'].float().contiguous()
        self.octree_children = states['voxel_octree_children_idx'].int().contiguous()
        self.centers = states['voxel_center_xyz'].float().contiguous()
        self.feats = states['voxel_vertex_idx'].int().contiguous()
        self.values = states['voxel_vertex_emb'].detach().float().contiguous()
        self.field = field
        self.mlp = TensorCoreMLP(field)
        bg = field.bg_color.bg_color.detach().float().cpu()
        self.bg = (ctypes.c_float * 3)(*bg.tolist())
        self.bg_depth = float(field.bg_color.depth)
        self.device = self.centers.device

    def mlp_fp8(self, n_calibration=65536, seed=0):
        """The tensor-core MLP with E4M3 hidden layers, its activation scales
        calibrated once on `n_calibration` points drawn uniformly inside
        random voxels of this scene (FP32 interpolation + FP32 MLP)."""
        if self.mlp.fp8 is None:
            g = torch.Generator(device="cpu").manual_seed(seed)
            V = self.centers.size(0)
            vox = torch.randint(0, V, (n_calibration,), generator=g).to(self.device)
            off = (torch.rand(n_calibration, 3, generator=g) - 0.5).to(self.device) * self.voxel_size
            xyz = self.centers[vox] + off
            emb = trilinear_embed(vox.int(), xyz, self.centers, self.feats, self.values,
                                  self.voxel_size)
            self.mlp.enable_fp8(emb)
        return self.mlp

    def bytes(self):
        ts = [self.octree_centers, self.octree_children, self.centers, self.feats, self.values]
        ts += self.mlp.w + self.mlp.b
        return sum(t.numel() * t.element_size() for t in ts)


# Sample capacity of a frame's first render, per ray; a frame that needs more
# is composited again with room for all its samples, and the capacity stays.
INITIAL_SAMPLES_PER_RAY = 32


def _frame_buffers(scene, R, stream):
    """Device buffers of the chain for frames of R rays on `stream`, kept on
    the scene and reused while the frame size stays the same. Keyed by stream:
    frames on one stream reuse them in stream order, frames on different
    streams never share them."""
    frames = scene.__dict__.setdefault("_frames", {})
    b = frames.get(stream)
    if b is not None and b["R"] == R:
        return b
    frames.pop(stream, None)
    dev, H = scene.device, scene.max_hits
    i32, i64 = torch.int32, torch.int64

    def e(*shape, dtype=torch.float32):
        return torch.empty(*shape, dtype=dtype, device=dev)

    b = {"R": R, "ro": e(R, 3), "idx": e(R, H, dtype=i32), "lo": e(R, H), "hi": e(R, H),
         "hits": e(R, dtype=torch.uint8), "scan": e(R, dtype=i32), "pix": e(R, dtype=i64),
         "n_hit": e(1, dtype=i64), "I": e(R, H, dtype=i32), "L": e(R, H), "U": e(R, H),
         "probs": e(R, H), "steps": e(R), "count": e(R, dtype=i32),
         "offset": torch.zeros(R + 1, dtype=i64, device=dev),
         "ws": ext._svo_workspace(1, scene.octree_centers.shape[0], dev),
         "bg": torch.tensor(list(scene.bg), dtype=torch.float32, device=dev),
         "err": torch.zeros(1, dtype=i32, device=dev),
         "counts_host": torch.zeros(2, dtype=i64).pin_memory(),
         "err_host": torch.zeros(1, dtype=i32).pin_memory(), "cap": 0}
    frames[stream] = b
    return b


def _sample_buffers(b, cap):
    """Compacted-sample buffers (voxel, xyz + distance, depth, field output)
    with room for at least `cap` samples, grown by a quarter when a frame
    needs more."""
    if cap > b["cap"]:
        cap = cap + cap // 4
        dev = b["ro"].device
        b["vox"] = b["xyzd"] = b["depth"] = b["field"] = None
        b["vox"] = torch.empty(cap, dtype=torch.int32, device=dev)
        b["xyzd"] = torch.empty(cap, 4, dtype=torch.float32, device=dev)
        b["depth"] = torch.empty(cap, dtype=torch.float32, device=dev)
        b["field"] = torch.empty(cap, 4, dtype=torch.float32, device=dev)
        b["cap"] = cap
    return b["vox"], b["xyzd"], b["depth"], b["field"]


def _compact(scene, b, R, ro, rd, cap, vox, xyzd, depth, err, stream):
    dev = scene.device
    with ext._timed("sample_compact", dev):
        check(LIB.nsvf_sample_compact_dev(R, _p(b["n_hit"]), scene.max_hits, _p(b["I"]), _p(b["L"]),
                                          _p(b["U"]), _p(b["probs"]), _p(b["steps"]), _p(ro), 3,
                                          _p(rd), _p(b["pix"]), _p(b["offset"]), cap, _p(vox),
                                          _p(xyzd), _p(depth), err, stream), "sample_compact_dev")


def _samples_on_device(scene, b, R, ro, rd, out, mlp, kahan, stream):
    """Steps 4-6 with the hit-ray and sample counts on the device only: the
    sample buffers have the frame buffers' capacity (INITIAL_SAMPLES_PER_RAY at
    first), and the host reads the counts and the error bits once, at the
    end. A frame with more samples than the capacity (error bit 1) is
    composited again with room for all of them."""
    dev = scene.device
    err = b["err"]
    counts, err_h = b["counts_host"], b["err_host"]
    cap = max(b["cap"], INITIAL_SAMPLES_PER_RAY * R)
    for _ in range(2):
        vox, xyzd, depth, field = _sample_buffers(b, cap)
        cap = b["cap"]
        err.zero_()
        _compact(scene, b, R, ro, rd, cap, vox, xyzd, depth, _p(err), stream)
        ns_dev = _p(b["offset"][R:])
        common = (_p(vox), _p(xyzd), scene.centers.size(0), scene.values.size(0), scene.voxel_size,
                  _p(scene.centers), _p(scene.feats), _p(scene.values))
        if mlp == "tc":
            m = scene.mlp
            with ext._timed("field_samples_bf16", dev):
                check(LIB.nsvf_field_samples_bf16_dev(cap, ns_dev, *common, m._wp, m._bp, _p(field),
                                                      _p(err), stream), "field_samples_bf16_dev")
        else:
            m = scene.mlp_fp8()
            with ext._timed("field_samples_fp8", dev):
                check(LIB.nsvf_field_samples_fp8_dev(cap, ns_dev, *common, m.fp8["wp"], m._bp,
                                                     m.fp8["scales"], _p(field), _p(err), stream),
                      "field_samples_fp8_dev")
        with ext._timed("composite_segments", dev):
            check(LIB.nsvf_composite_segments_dev(
                R, _p(b["n_hit"]), _p(b["offset"]), cap, _p(field), _p(xyzd), _p(depth), _p(b["pix"]),
                7.0, scene.bg, scene.bg_depth, _p(out["colors"]), _p(out["depths"]),
                _p(out["missed"]), int(bool(kahan)), stream), "composite_segments_dev")
        counts[0:1].copy_(b["n_hit"], non_blocking=True)
        counts[1:2].copy_(b["offset"][R:], non_blocking=True)
        err_h.copy_(err, non_blocking=True)
        torch.cuda.current_stream(dev).synchronize()
        n, ns, e = int(counts[0]), int(counts[1]), int(err_h[0])
        if not (e & 2):
            break
        cap = ns
    if e & ~2:
        ext.error_word(dev).bitwise_or_(err)
    out["n_hit_rays"], out["n_samples"] = n, ns
    return out


def render_frame(scene, ray_start, ray_dir, kahan=True, out=None, mlp="tc"):
    """ray_start [3] (shared origin) or [R, 3], ray_dir [R, 3] (FP32, on the
    scene's device) -> dict(colors [R, 3], depths [R], missed [R],
    n_hit_rays, n_samples).
    mlp: "tc" (interpolation fused into the tcgen05 BF16 MLP), "tc_fp8" (the
    same with E4M3 hidden layers), "tc_unfused" (interpolation kernel, then
    the MLP kernel), "bf16_emulated" / "fp8_emulated" (torch emulations of
    the kernels' rounding) or "fp32" (the field's FP32 torch forward). The
    two tensor-core modes run on device-side counts with one host read at
    the end of the frame; the others read the sample count mid-frame to size
    their torch tensors."""
    dev = scene.device
    R = ray_dir.shape[0]
    if out is None:
        out = {"colors": torch.empty(R, 3, device=dev), "depths": torch.empty(R, device=dev),
               "missed": torch.empty(R, device=dev)}
    out["n_hit_rays"] = out["n_samples"] = 0
    if R == 0:
        return out
    H = scene.max_hits
    stream = ext.ctypes_stream(dev)
    b = _frame_buffers(scene, R, stream)
    rd = ray_dir.float().contiguous()
    if ray_start.dim() == 1:
        ro = b["ro"]
        ro.copy_(ray_start.float().reshape(1, 3).expand(R, 3))
    else:
        ro = ray_start.float().contiguous()
    err = _p(ext.error_word(dev))
    n_nodes = scene.octree_centers.shape[0]
    with ext._timed("svo_intersect_sorted", dev):
        check(LIB.nsvf_svo_intersect_sorted(1, 1, n_nodes, R, scene.voxel_size, H, _p(ro), _p(rd),
                                            _p(scene.octree_centers), _p(scene.octree_children),
                                            _p(b["idx"]), _p(b["lo"]), _p(b["hi"]), _p(b["hits"]),
                                            err, _p(b["ws"]), stream), "svo_intersect_sorted")
    with ext._timed("hit_rows", dev):
        torch.cumsum(b["hits"], 0, dtype=torch.int32, out=b["scan"])
        check(LIB.nsvf_compact_hits(R, _p(b["hits"]), _p(b["scan"]), _p(b["pix"]), _p(b["n_hit"]),
                                    stream), "compact_hits")
        check(LIB.nsvf_gather_probs(R, _p(b["n_hit"]), H, scene.step_size, _p(b["pix"]),
                                    _p(b["idx"]), _p(b["lo"]), _p(b["hi"]), _p(b["I"]), _p(b["L"]),
                                    _p(b["U"]), _p(b["probs"]), _p(b["steps"]), stream),
              "gather_probs")
    with ext._timed("sample_count", dev):
        check(LIB.nsvf_sample_count_dev(R, _p(b["n_hit"]), H, _p(b["I"]), _p(b["L"]), _p(b["U"]),
                                        _p(b["probs"]), _p(b["steps"]), _p(b["count"]), stream),
              "sample_count_dev")
    offset = b["offset"]
    torch.cumsum(b["count"], 0, out=offset[1:])
    out["colors"].copy_(b["bg"].expand(R, 3))
    out["depths"].fill_(scene.bg_depth)
    out["missed"].fill_(1.0)
    if mlp in ("tc", "tc_fp8"):
        return _samples_on_device(scene, b, R, ro, rd, out, mlp, kahan, stream)
    counts = b["counts_host"]
    counts[0:1].copy_(b["n_hit"], non_blocking=True)
    counts[1:2].copy_(offset[R:], non_blocking=True)
    torch.cuda.current_stream(dev).synchronize()
    n, ns = int(counts[0]), int(counts[1])
    out["n_hit_rays"], out["n_samples"] = n, ns
    if n == 0:
        return out
    vox, xyzd, depth, _ = _sample_buffers(b, ns)
    vox, xyzd, depth = vox[:ns], xyzd[:ns], depth[:ns]
    _compact(scene, b, R, ro, rd, ns, vox, xyzd, depth, err, stream)
    emb = trilinear_embed(vox, xyzd[:, :3], scene.centers, scene.feats, scene.values,
                          scene.voxel_size)
    if mlp == "tc_unfused":
        field = scene.mlp(emb)
    elif mlp == "bf16_emulated":
        field = scene.mlp.reference_bf16(emb).contiguous()
    elif mlp == "fp8_emulated":
        field = scene.mlp_fp8().reference_fp8(emb).contiguous()
    elif mlp == "fp32":
        field = scene.field.mlp(emb).float().contiguous()
    else:
        raise ValueError("unknown mlp mode %r" % (mlp,))
    with ext._timed("composite_segments", dev):
        check(LIB.nsvf_composite_segments(
            n, _p(offset), _p(field), _p(xyzd), _p(depth), _p(b["pix"]), 7.0, scene.bg,
            scene.bg_depth, _p(out["colors"]), _p(out["depths"]), _p(out["missed"]),
            int(bool(kahan)), stream), "composite_segments")
    return out
