"""Served frame renderer: the hot path as a short chain of sm_103a kernels.

For one frame of rays of a resident scene:

1. nsvf_svo_intersect_grid    -- the octree's hit lists in depth order from a
   sweep over the leaf grid (FP32, exact; nsvf_svo_intersect_sorted, the
   depth-first traversal + sort, for trees not in leaf-grid form)
2. nsvf_compact_hits          -- order-preserving compaction of the hit rays
   (on a torch prefix sum of the hit flags)
3. nsvf_gather_probs          -- the hit rays' lists and their sampling
   distribution (fairnr/models/nsvf.py:65-74), warp per ray
4. nsvf_sample_scan_compact_dev -- the inverse-CDF walk (deterministic
   jitter, the reference's launch layout) writing only the valid samples,
   compacted per ray: counts, their prefix sum and the samples in one pass
   (nsvf_sample_count_dev, a prefix sum and nsvf_sample_compact_dev where
   the host needs the sample count before the field runs)
5. nsvf_field_samples_bf16    -- corner-embedding interpolation fused into the
                                 tcgen05 BF16 field MLP (FP32 accumulation);
                                 embeddings and activations stay on chip
6. nsvf_composite_segments    -- compensated transmittance compositing into
                                 the frame (the background is filled first)

With the tensor-core field the whole chain runs on device-side counts (hit
rays, samples), so the host enqueues the frame while the traversal runs and
reads the counts once, at the end. The sample buffers keep a capacity across
frames; a frame that needs more is composited again with room for it.

Samples far outside their voxel (the reference's inverse-CDF tail can give a
sample the voxel id of the next hit slot, fairnr/clib/src/sample_gpu.cu:
188-201) are listed by the MLP's loaders and their field is evaluated again in
double-float arithmetic (nsvf_field_exact_dev) before compositing: their
extrapolated trilinear weights would turn BF16 rounding into colour errors of
units.

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


def _is_tensor_core_field(field):
    layers = getattr(field, "layers", None)
    if layers is None or not hasattr(field, "mlp"):
        return False
    dims = [(getattr(l, "out_features", None), getattr(l, "in_features", None)) for l in layers]
    return dims == [(128, 32), (128, 128), (128, 128), (128, 128), (4, 128)]


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
        # the leaf-grid form of the octree (host-built once per scene); trees
        # not in that form go through the depth-first kernel
        self.svo_grid = ext.SvoGrid(self.octree_centers, self.octree_children, self.voxel_size)
        self.centers = states['voxel_center_xyz'].float().contiguous()
        self.feats = states['voxel_vertex_idx'].int().contiguous()
        self.values = states['voxel_vertex_emb'].detach().float().contiguous()
        self.field = field
        self.device = self.centers.device
        # The tensor-core MLP takes the workloads' 4 x 128 ReLU field; any
        # other field of the reference's field interface (a checkpointed
        # radiance field, field.RaidanceField) renders through the served
        # chain with its own FP32 torch modules (render_frame(mlp="field")).
        self.mlp = TensorCoreMLP(field) if _is_tensor_core_field(field) else None
        if self.mlp is not None:
            # BF16 bias correction, calibrated once per scene
            self.mlp.calibrate_bias(self.calibration_emb())
        bg = field.bg_color.bg_color.detach().float().cpu()
        self.bg = (ctypes.c_float * 3)(*bg.tolist())
        self.bg_depth = float(field.bg_color.depth)

    def calibration_emb(self, n=65536, seed=0):
        """FP32 embeddings of `n` points drawn uniformly inside random voxels
        of this scene (seeded): the calibration set of the BF16 bias
        correction and of the FP8 activation scales."""
        g = torch.Generator(device="cpu").manual_seed(seed)
        V = self.centers.size(0)
        vox = torch.randint(0, V, (n,), generator=g).to(self.device)
        off = (torch.rand(n, 3, generator=g) - 0.5).to(self.device) * self.voxel_size
        xyz = self.centers[vox] + off
        return trilinear_embed(vox.int(), xyz, self.centers, self.feats, self.values,
                               self.voxel_size)

    def mlp_fp8(self, n_calibration=65536, seed=0):
        """The tensor-core MLP with E4M3 hidden layers, its activation scales
        calibrated once on `n_calibration` points drawn uniformly inside
        random voxels of this scene (FP32 interpolation + FP32 MLP)."""
        if self.mlp.fp8 is None:
            self.mlp.enable_fp8(self.calibration_emb(n_calibration, seed))
        return self.mlp

    def bytes(self):
        ts = [self.octree_centers, self.octree_children, self.centers, self.feats, self.values]
        if self.mlp is not None:
            ts += self.mlp.w + self.mlp.b
        else:
            ts += [t for t in self.field.parameters()]
        return sum(t.numel() * t.element_size() for t in ts) + self.svo_grid.bytes()


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
         "scan_ws": torch.empty(int(LIB.nsvf_sample_scan_bytes(R)), dtype=torch.uint8, device=dev),
         "ws": ext._svo_workspace(1, scene.octree_centers.shape[0], dev),
         "bg": torch.tensor(list(scene.bg), dtype=torch.float32, device=dev),
         "err": torch.zeros(1, dtype=i32, device=dev),
         "counts_host": torch.zeros(4, dtype=i64).pin_memory(),
         "err_host": torch.zeros(1, dtype=i32).pin_memory(), "cap": 0,
         "n_outl": torch.zeros(1, dtype=i64, device=dev), "outl": None, "outl_cap": 0,
         "n_refine": torch.zeros(1, dtype=i64, device=dev)}
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


# Initial capacity of the list of samples far outside their voxel (about
# 1.2k per c2 frame, 2.3k per c4 frame); it grows when a frame needs more.
INITIAL_OUTLIERS = 16384


# A ray whose far-outside sample has a colour magnitude above this gets its
# other samples evaluated in FP32 (nsvf_field_refine_fp32_dev): the BF16 error
# of the transmittance in front of that sample, about 1e-6 with the bias
# correction on the c4 frame, times the colour stays below ~1e-3 elsewhere.
REFINE_ABOVE = 1000.0


def _outlier_list(b, cap):
    if cap > b["outl_cap"]:
        b["outl"] = None
        b["outl"] = torch.empty(2 * cap, dtype=torch.int64, device=b["ro"].device)
        b["outl_cap"] = cap
    return b["outl"], b["outl_cap"]


def _exact_pass(scene, b, R, ro, rd, vox, xyzd, depth, field, err, stream, cap, refine=True):
    """nsvf_field_exact_dev over the frame's outlier list: the listed samples'
    field in double-float, written over `field`; then the rays whose listed
    sample's colour exceeds REFINE_ABOVE get their other samples in FP32
    (nsvf_field_refine_fp32_dev). The second half of the outlier buffer holds
    those rays."""
    m = scene.mlp
    ocap = b["outl_cap"]
    rows = b["outl"][ocap:]
    b["n_refine"].zero_()
    with ext._timed("field_exact", scene.device):
        check(LIB.nsvf_field_exact_dev(R, _p(b["n_hit"]), _p(b["offset"]), _p(b["pix"]), _p(ro), 3,
                                       _p(rd), _p(depth), _p(vox), scene.centers.size(0),
                                       scene.values.size(0), scene.voxel_size, _p(scene.centers),
                                       _p(scene.feats), _p(scene.values), m._wtp, m._bp,
                                       _p(b["outl"]), _p(b["n_outl"]), ocap, _p(field),
                                       REFINE_ABOVE, _p(rows) if refine else None,
                                       _p(b["n_refine"]) if refine else None, ocap, err,
                                       stream), "field_exact_dev")
    if not refine:
        return
    with ext._timed("field_refine_fp32", scene.device):
        check(LIB.nsvf_field_refine_fp32_dev(_p(rows), _p(b["n_refine"]), ocap, R, _p(b["n_hit"]),
                                             _p(b["offset"]), cap, _p(vox), _p(xyzd),
                                             scene.centers.size(0), scene.values.size(0),
                                             scene.voxel_size, _p(scene.centers), _p(scene.feats),
                                             _p(scene.values), m._wtp, m._bp, _p(field), stream),
              "field_refine_fp32_dev")


def _scan_compact(scene, b, R, ro, rd, cap, vox, xyzd, depth, err, stream):
    """Counts, offsets and samples of the hit rays in one pass."""
    dev = scene.device
    with ext._timed("sample_scan_compact", dev):
        check(LIB.nsvf_sample_scan_compact_dev(
            R, _p(b["n_hit"]), scene.max_hits, _p(b["I"]), _p(b["L"]), _p(b["U"]), _p(b["probs"]),
            _p(b["steps"]), _p(ro), 3, _p(rd), _p(b["pix"]), _p(b["offset"]), cap, _p(vox),
            _p(xyzd), _p(depth), _p(b["scan_ws"]), b["scan_ws"].numel(), err, stream),
            "sample_scan_compact_dev")


def _compact(scene, b, R, ro, rd, cap, vox, xyzd, depth, err, stream):
    dev = scene.device
    with ext._timed("sample_compact", dev):
        check(LIB.nsvf_sample_compact_dev(R, _p(b["n_hit"]), scene.max_hits, _p(b["I"]), _p(b["L"]),
                                          _p(b["U"]), _p(b["probs"]), _p(b["steps"]), _p(ro), 3,
                                          _p(rd), _p(b["pix"]), _p(b["offset"]), cap, _p(vox),
                                          _p(xyzd), _p(depth), err, stream), "sample_compact_dev")


# Rows up to this many hit slots take the one-pass count + compaction.
SCAN_MAX_HITS = 128


def _count(scene, b, R, stream):
    """Per-hit-ray sample counts and their prefix sum into b["offset"]."""
    dev = scene.device
    with ext._timed("sample_count", dev):
        check(LIB.nsvf_sample_count_dev(R, _p(b["n_hit"]), scene.max_hits, _p(b["I"]), _p(b["L"]),
                                        _p(b["U"]), _p(b["probs"]), _p(b["steps"]), _p(b["count"]),
                                        stream), "sample_count_dev")
    torch.cumsum(b["count"], 0, out=b["offset"][1:])


def _samples_on_device(scene, b, R, ro, rd, out, mlp, kahan, exact, stream):
    """Steps 4-6 with the hit-ray and sample counts on the device only: the
    sample buffers have the frame buffers' capacity (INITIAL_SAMPLES_PER_RAY at
    first), and the host reads the counts and the error bits once, at the
    end. A frame with more samples than the capacity (error bit 1), or more
    samples far outside their voxel than the outlier list holds (bit 4), is
    composited again with room for all of them."""
    dev = scene.device
    err = b["err"]
    counts, err_h = b["counts_host"], b["err_host"]
    cap = max(b["cap"], INITIAL_SAMPLES_PER_RAY * R)
    ocap = max(b["outl_cap"], INITIAL_OUTLIERS)
    for _ in range(3):
        vox, xyzd, depth, field = _sample_buffers(b, cap)
        cap = b["cap"]
        outl, ocap = _outlier_list(b, ocap) if exact else (None, 0)
        n_outl = b["n_outl"] if exact else None
        err.zero_()
        if exact:
            n_outl.zero_()
        if scene.max_hits <= SCAN_MAX_HITS:
            _scan_compact(scene, b, R, ro, rd, cap, vox, xyzd, depth, _p(err), stream)
        else:
            _count(scene, b, R, stream)
            _compact(scene, b, R, ro, rd, cap, vox, xyzd, depth, _p(err), stream)
        ns_dev = _p(b["offset"][R:])
        common = (_p(vox), _p(xyzd), scene.centers.size(0), scene.values.size(0), scene.voxel_size,
                  _p(scene.centers), _p(scene.feats), _p(scene.values))
        if mlp == "tc":
            m = scene.mlp
            with ext._timed("field_samples_bf16", dev):
                check(LIB.nsvf_field_samples_bf16_dev(cap, ns_dev, *common, m._wp, m._bp_tc,
                                                      _p(field), _p(outl), _p(n_outl), ocap,
                                                      _p(err), stream), "field_samples_bf16_dev")
        else:
            m = scene.mlp_fp8()
            with ext._timed("field_samples_fp8", dev):
                check(LIB.nsvf_field_samples_fp8_dev(cap, ns_dev, *common, m.fp8["wp"], m._bp,
                                                     m.fp8["scales"], _p(field), _p(outl),
                                                     _p(n_outl), ocap, _p(err), stream),
                      "field_samples_fp8_dev")
        if exact:
            _exact_pass(scene, b, R, ro, rd, vox, xyzd, depth, field, _p(err), stream, cap)
        with ext._timed("composite_segments", dev):
            check(LIB.nsvf_composite_segments_dev(
                R, _p(b["n_hit"]), _p(b["offset"]), cap, _p(field), _p(xyzd), _p(depth), _p(b["pix"]),
                7.0, scene.bg, scene.bg_depth, _p(out["colors"]), _p(out["depths"]),
                _p(out["missed"]), int(bool(kahan)), stream), "composite_segments_dev")
        counts[0:1].copy_(b["n_hit"], non_blocking=True)
        counts[1:2].copy_(b["offset"][R:], non_blocking=True)
        if exact:
            counts[2:3].copy_(n_outl, non_blocking=True)
            counts[3:4].copy_(b["n_refine"], non_blocking=True)
        err_h.copy_(err, non_blocking=True)
        torch.cuda.current_stream(dev).synchronize()
        n, ns, e = int(counts[0]), int(counts[1]), int(err_h[0])
        n_far = int(counts[2]) if exact else 0
        n_ref = int(counts[3]) if exact else 0
        if not (e & (2 | 16)):
            break
        if e & 2:
            cap = ns
        if e & 16:
            ocap = max(n_far, n_ref) + max(n_far, n_ref) // 4
    if e & ~(2 | 16):
        ext.error_word(dev).bitwise_or_(err)
    out["n_hit_rays"], out["n_samples"], out["n_far_outside"] = n, ns, n_far
    out["n_rays_refined_fp32"] = n_ref
    return out


def render_frame(scene, ray_start, ray_dir, kahan=True, out=None, mlp="tc", exact=True,
                 traversal="grid"):
    """ray_start [3] (shared origin) or [R, 3], ray_dir [R, 3] (FP32, on the
    scene's device) -> dict(colors [R, 3], depths [R], missed [R],
    n_hit_rays, n_samples, n_far_outside).
    exact: samples far outside their voxel (a trilinear coordinate outside
    [-0.5, 1.5]; the reference's sampling tail gives about one per thousand
    hit rays) get their field evaluated again in double-float arithmetic
    (nsvf_field_exact_dev) before compositing, whatever `mlp` computed.
    mlp: "tc" (interpolation fused into the tcgen05 BF16 MLP), "tc_fp8" (the
    same with E4M3 hidden layers), "tc_unfused" (interpolation kernel, then
    the MLP kernel), "bf16_emulated" / "fp8_emulated" (torch emulations of
    the kernels' rounding), "fp32" (the 4 x 128 field's FP32 torch forward)
    or "field" (any field with the reference's field interface, e.g. a
    checkpointed field.RaidanceField: its FP32 torch forward on the samples'
    embeddings, positions and ray directions; the default for scenes whose
    field the tensor-core MLP does not take). The
    two tensor-core modes run on device-side counts with one host read at
    the end of the frame; the others read the sample count mid-frame to size
    their torch tensors.
    traversal: "grid" (the leaf-grid sweep, nsvf_svo_intersect_grid, where the
    scene's octree is in leaf-grid form) or "dfs" (the depth-first kernel,
    nsvf_svo_intersect_sorted); both give the same hit lists bit for bit."""
    dev = scene.device
    R = ray_dir.shape[0]
    if scene.mlp is None and mlp != "field":
        if mlp != "tc":
            raise ValueError("mlp=%r needs the 4 x 128 field; this scene's field renders with "
                             "mlp='field'" % (mlp,))
        mlp = "field"
    if out is None:
        out = {"colors": torch.empty(R, 3, device=dev), "depths": torch.empty(R, device=dev),
               "missed": torch.empty(R, device=dev)}
    out["n_hit_rays"] = out["n_samples"] = out["n_far_outside"] = out["n_rays_refined_fp32"] = 0
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
    if traversal == "grid" and scene.svo_grid.ok:
        with ext._timed("svo_intersect_grid", dev):
            # rows end at their first -1: nsvf_gather_probs reads no further
            scene.svo_grid.intersect_into(R, H, _p(ro), _p(rd), _p(b["idx"]), _p(b["lo"]),
                                          _p(b["hi"]), _p(b["hits"]), stream, padded=False)
    else:
        with ext._timed("svo_intersect_sorted", dev):
            check(LIB.nsvf_svo_intersect_sorted(1, 1, n_nodes, R, scene.voxel_size, H, _p(ro),
                                                _p(rd), _p(scene.octree_centers),
                                                _p(scene.octree_children), _p(b["idx"]),
                                                _p(b["lo"]), _p(b["hi"]), _p(b["hits"]), err,
                                                _p(b["ws"]), stream), "svo_intersect_sorted")
    with ext._timed("hit_rows", dev):
        torch.cumsum(b["hits"], 0, dtype=torch.int32, out=b["scan"])
        check(LIB.nsvf_compact_hits(R, _p(b["hits"]), _p(b["scan"]), _p(b["pix"]), _p(b["n_hit"]),
                                    stream), "compact_hits")
        check(LIB.nsvf_gather_probs(R, _p(b["n_hit"]), H, scene.step_size, _p(b["pix"]),
                                    _p(b["idx"]), _p(b["lo"]), _p(b["hi"]), _p(b["I"]), _p(b["L"]),
                                    _p(b["U"]), _p(b["probs"]), _p(b["steps"]), stream),
              "gather_probs")
    out["colors"].copy_(b["bg"].expand(R, 3))
    out["depths"].fill_(scene.bg_depth)
    out["missed"].fill_(1.0)
    if mlp in ("tc", "tc_fp8"):
        return _samples_on_device(scene, b, R, ro, rd, out, mlp, kahan, exact, stream)
    _count(scene, b, R, stream)
    offset = b["offset"]
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
        # (the emulation uses the BF16 kernels' corrected biases)
        field = scene.mlp.reference_bf16(emb).contiguous()
    elif mlp == "fp8_emulated":
        field = scene.mlp_fp8().reference_fp8(emb).contiguous()
    elif mlp == "fp32":
        field = scene.field.mlp(emb).float().contiguous()
    elif mlp == "field":
        field = _field_forward(scene, b, n, ns, ro, rd, offset, vox, xyzd, emb)
        # the field runs in FP32 like the reference's; the double-float pass
        # is specific to the 4 x 128 field
        exact = False
    else:
        raise ValueError("unknown mlp mode %r" % (mlp,))
    if exact:
        ocap = max(b["outl_cap"], INITIAL_OUTLIERS)
        for _ in range(2):
            outl, ocap = _outlier_list(b, ocap)
            b["n_outl"].zero_()
            with ext._timed("flag_outliers", dev):
                check(LIB.nsvf_flag_outliers(ns, None, _p(vox), _p(xyzd), scene.centers.size(0),
                                             scene.voxel_size, _p(scene.centers), _p(outl),
                                             _p(b["n_outl"]), ocap, None, stream), "flag_outliers")
            n_far = int(b["n_outl"].item())
            if n_far <= ocap:
                break
            ocap = n_far + n_far // 4
        _exact_pass(scene, b, R, ro, rd, vox, xyzd, depth, field, err, stream, ns,
                    refine=mlp != "fp32")
        out["n_far_outside"] = n_far
        out["n_rays_refined_fp32"] = int(b["n_refine"].item())
    with ext._timed("composite_segments", dev):
        check(LIB.nsvf_composite_segments(
            n, _p(offset), _p(field), _p(xyzd), _p(depth), _p(b["pix"]), 7.0, scene.bg,
            scene.bg_depth, _p(out["colors"]), _p(out["depths"]), _p(out["missed"]),
            int(bool(kahan)), stream), "composite_segments")
    return out


# samples per call of a field module on the served path's generic mode
FIELD_CHUNK = 1 << 20


def _field_forward(scene, b, n, ns, ro, rd, offset, vox, xyzd, emb):
    """The scene's field module on the compacted samples, through the
    reference's field interface (inputs 'emb', 'pos', 'ray', 'dists';
    fairnr/modules/renderer.py:105-111), FIELD_CHUNK samples at a time (the
    reference's field forward builds an autograd graph for its normals):
    -> [ns, 4] (sigma, r, g, b)."""
    dev = scene.device
    counts = offset[1:n + 1] - offset[:n]
    rows = torch.repeat_interleave(torch.arange(n, device=dev), counts, output_size=ns)
    ray = rd[b["pix"][:n][rows]]
    out = torch.empty(ns, 4, dtype=torch.float32, device=dev)
    for s0 in range(0, ns, FIELD_CHUNK):
        s1 = min(ns, s0 + FIELD_CHUNK)
        inputs = {"emb": emb[s0:s1], "pos": xyzd[s0:s1, :3], "ray": ray[s0:s1],
                  "dists": xyzd[s0:s1, 3]}
        res = scene.field(inputs, outputs=("sigma", "texture"))
        out[s0:s1, 0] = res["sigma"].reshape(-1).detach().float()
        out[s0:s1, 1:4] = res["texture"].reshape(-1, 3).detach().float()
    return out


class HostFrames:
    """Frames whose rays sit in pinned host memory, rendered with their
    results returned to pinned host memory, the copies overlapped with the
    rendering: frame i + 1's rays go to the device on one copy stream while
    frame i renders, and frame i's colours and depths come back on a second
    copy stream while frame i + 1 renders. Two device slots per direction;
    events order every reuse of a slot after the copy or frame that last
    used it.

    render(frames) takes a sequence of (ray_start [3] or [R, 3], ray_dir
    [R, 3], colors [R, 3], depths [R]) host tensors (the last two pinned,
    written) and returns when every frame's results are in host memory.
    Frames have R rays each."""

    def __init__(self, scene, R, mlp="tc", kahan=True):
        dev = scene.device
        self.scene, self.R, self.mlp, self.kahan = scene, R, mlp, kahan
        self.copy_in = torch.cuda.Stream(dev)
        self.copy_out = torch.cuda.Stream(dev)
        e = lambda *s: torch.empty(*s, dtype=torch.float32, device=dev)
        self.ro = [None, None]
        self.rd = [e(R, 3), e(R, 3)]
        self.out = [{"colors": e(R, 3), "depths": e(R), "missed": e(R)} for _ in range(2)]
        ev = lambda: [torch.cuda.Event(), torch.cuda.Event()]
        self.in_ready, self.in_free, self.done, self.out_free = ev(), ev(), ev(), ev()
        self.n_samples = 0

    def _stage_in(self, i, ro_h, rd_h):
        s = i % 2
        if self.ro[s] is None or self.ro[s].shape != ro_h.shape:
            # a new origin buffer only after every use of the old one
            self.in_free[s].synchronize()
            self.ro[s] = torch.empty(ro_h.shape, dtype=torch.float32, device=self.scene.device)
        with torch.cuda.stream(self.copy_in):
            if i >= 2:
                self.copy_in.wait_event(self.in_free[s])
            self.ro[s].copy_(ro_h, non_blocking=True)
            self.rd[s].copy_(rd_h, non_blocking=True)
            self.in_ready[s].record(self.copy_in)

    def render(self, frames, before_frame=None):
        """before_frame(i), if given, runs on the rendering stream before
        frame i is enqueued (for example an L2 flush between timed frames)."""
        frames = list(frames)
        if not frames:
            return
        cur = torch.cuda.current_stream(self.scene.device)
        self._stage_in(0, frames[0][0], frames[0][1])
        for i, (_, rd_h, col_h, dep_h) in enumerate(frames):
            if rd_h.shape[0] != self.R:
                raise ValueError("frame %d has %d rays, the pipeline %d" % (i, rd_h.shape[0], self.R))
            if i + 1 < len(frames):
                self._stage_in(i + 1, frames[i + 1][0], frames[i + 1][1])
            s = i % 2
            if before_frame is not None:
                before_frame(i)
            cur.wait_event(self.in_ready[s])
            if i >= 2:
                cur.wait_event(self.out_free[s])
            out = render_frame(self.scene, self.ro[s], self.rd[s], kahan=self.kahan,
                               out=self.out[s], mlp=self.mlp)
            self.n_samples += int(out.get("n_samples", 0) or 0)
            self.in_free[s].record(cur)
            self.done[s].record(cur)
            with torch.cuda.stream(self.copy_out):
                self.copy_out.wait_event(self.done[s])
                col_h.copy_(out["colors"], non_blocking=True)
                dep_h.copy_(out["depths"], non_blocking=True)
                self.out_free[s].record(self.copy_out)
        self.copy_out.synchronize()
