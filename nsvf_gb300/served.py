"""Served frame renderer: the hot path as a short chain of sm_103a kernels.

For one frame of rays of a resident scene:

1. nsvf_svo_intersect_sorted  -- octree traversal + depth sort (FP32, exact)
2. hit-ray compaction, probs/steps (fairnr/models/nsvf.py:65-74, torch)
3. nsvf_sample_count / nsvf_sample_compact -- the inverse-CDF walk
   (deterministic jitter, the reference's launch layout) writing only the
   valid samples, compacted per ray
4. nsvf_field_samples_bf16    -- corner-embedding interpolation fused into the
                                 tcgen05 BF16 field MLP (FP32 accumulation);
                                 embeddings and activations stay on chip
6. nsvf_composite_segments    -- compensated transmittance compositing and
                                 the background fill, straight into the frame

Geometry (slab distances, sample depths and positions) stays FP32 and is the
same as the drop-in path's; only the MLP runs in BF16. Two host
synchronisations per frame read the hit count and the sample count.
"""
import ctypes

import torch

from . import ext
from ._lib import LIB, check
from .clib import inverse_cdf_layout
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


def render_frame(scene, ray_start, ray_dir, kahan=True, out=None, mlp="tc"):
    """ray_start [3] (shared origin) or [R, 3], ray_dir [R, 3] (FP32, on the
    scene's device) -> dict(colors [R, 3], depths [R], missed [R]).
    mlp: "tc" (interpolation fused into the tcgen05 BF16 MLP), "tc_fp8" (the
    same with E4M3 hidden layers), "tc_unfused" (interpolation kernel, then
    the MLP kernel), "bf16_emulated" / "fp8_emulated" (torch emulations of
    the kernels' rounding) or "fp32" (the field's FP32 torch forward)."""
    dev = scene.device
    R = ray_dir.shape[0]
    rd = ray_dir.float().contiguous()
    shared_origin = ray_start.dim() == 1
    ro = ray_start.float().reshape(1, 3).expand(R, 3).contiguous() if shared_origin \
        else ray_start.float().contiguous()
    if out is None:
        out = {"colors": torch.empty(R, 3, device=dev), "depths": torch.empty(R, device=dev),
               "missed": torch.empty(R, device=dev)}
    bg = torch.tensor(list(scene.bg), device=dev)
    out["colors"].copy_(bg.expand(R, 3))
    out["depths"].fill_(scene.bg_depth)
    out["missed"].fill_(1.0)
    H = scene.max_hits
    idx, lo, hi, hits = ext.svo_intersect_sorted(
        ro.view(1, R, 3), rd.view(1, R, 3), scene.octree_centers.unsqueeze(0),
        scene.octree_children.unsqueeze(0), scene.voxel_size, H)
    idx, lo, hi, hits = idx[0], lo[0], hi[0], hits[0]
    pix = hits.nonzero().squeeze(1)
    n = pix.numel()
    if n == 0:
        return out
    I, L, Hh = idx[pix].contiguous(), lo[pix].contiguous(), hi[pix].contiguous()
    d = (Hh - L).masked_fill(I.eq(-1), 0)
    tot = d.sum(-1, keepdim=True)
    probs = (d / tot).contiguous()
    steps = (tot[:, 0] / scene.step_size).contiguous()
    layout = torch.tensor(inverse_cdf_layout(n), dtype=torch.int64)
    count = torch.empty(n, dtype=torch.int32, device=dev)
    stream = ext.ctypes_stream(dev)
    with ext._timed("sample_count", dev):
        check(LIB.nsvf_sample_count(n, H, _p(I), _p(L), _p(Hh), _p(probs), _p(steps),
                                    layout.data_ptr(), _p(count), stream), "sample_count")
    offset = torch.zeros(n + 1, dtype=torch.int64, device=dev)
    torch.cumsum(count, 0, out=offset[1:])
    ns = int(offset[-1].item())
    vox = torch.empty(ns, dtype=torch.int32, device=dev)
    xyzd = torch.empty(ns, 4, dtype=torch.float32, device=dev)
    depth = torch.empty(ns, dtype=torch.float32, device=dev)
    ro_h = ro[pix].contiguous()
    rd_h = rd[pix].contiguous()
    with ext._timed("sample_compact", dev):
        check(LIB.nsvf_sample_compact(n, H, _p(I), _p(L), _p(Hh), _p(probs), _p(steps),
                                      layout.data_ptr(), _p(ro_h), 3, _p(rd_h), _p(offset),
                                      _p(vox), _p(xyzd), _p(depth), _p(ext.error_word(dev)),
                                      stream), "sample_compact")
    if mlp == "tc":
        field = scene.mlp.field_samples(vox, xyzd, scene.centers, scene.feats, scene.values,
                                        scene.voxel_size)
    elif mlp == "tc_fp8":
        field = scene.mlp_fp8().field_samples_fp8(vox, xyzd, scene.centers, scene.feats,
                                                  scene.values, scene.voxel_size)
    else:
        emb = trilinear_embed(vox, xyzd[:, :3], scene.centers, scene.feats, scene.values,
                              scene.voxel_size)
        if mlp == "tc_unfused":
            field = scene.mlp(emb)
        elif mlp == "bf16_emulated":
            field = scene.mlp.reference_bf16(emb).contiguous()
        elif mlp == "fp8_emulated":
            field = scene.mlp_fp8().reference_fp8(emb).contiguous()
        else:
            field = scene.field.mlp(emb).float().contiguous()
    with ext._timed("composite_segments", dev):
        check(LIB.nsvf_composite_segments(
            n, _p(offset), _p(field), _p(xyzd), _p(depth), _p(pix), 7.0, scene.bg,
            scene.bg_depth, _p(out["colors"]), _p(out["depths"]), _p(out["missed"]),
            int(bool(kahan)), stream), "composite_segments")
    out["n_hit_rays"] = n
    out["n_samples"] = ns
    return out
