"""The double-float pass over samples far outside their voxel
(nsvf_field_exact_dev) on the full 800x800 c2 frame.

The reference's inverse-CDF tail (fairnr/clib/src/sample_gpu.cu:188-201) can
give a sample the voxel id of the next hit slot; its trilinear weights then
extrapolate and the field there is thousands. The served chain lists such
samples in the tensor-core loaders and evaluates them again in double-float
arithmetic. Checked here: the loaders' list equals the standalone flag
kernel's, and each re-evaluated (sigma, r, g, b) equals a float64 evaluation
of the same sample (position from the same FP32 ray and depth) to FP32
rounding."""
import argparse

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _c2(dev, voxel=1.0 / 64):
    from nsvf_gb300 import scenes
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    p, vs = scenes.scene_shell(voxel)
    args = argparse.Namespace(voxel_size=vs, max_hits=64, raymarching_stepsize_ratio=0.125,
                              voxel_embed_dim=32, use_octree=True, deterministic_step=True,
                              chunk_size=64)
    enc = SparseVoxelEncoder(args, points=p)
    with torch.no_grad():
        enc.values.weight.copy_(scenes.voxel_embeddings(enc.values.weight.shape[0], 32, 0.01, seed=1))
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=2))
    return enc.to(dev).eval(), field.to(dev).eval(), vs


def _float64_field(scene, ro, rd, depth, vox, pix, offset, n_hit, sel, field):
    """(sigma, r, g, b) in float64 at samples `sel` of the served buffers."""
    dev = ro.device
    off = offset[:n_hit + 1]
    row = torch.searchsorted(off, sel, right=True) - 1
    ray = pix[row]
    t = depth[sel].double()
    xyz = ro[ray].double() + rd[ray].double() * t[:, None]
    v = vox[sel].long()
    c = scene.centers.double()[v]
    p = ((xyz - c) / float(scene.voxel_size) + 0.5)[:, None, :]
    cc = torch.tensor([-1.0, 1.0], dtype=torch.float64, device=dev)
    ox, oy, oz = torch.meshgrid([cc, cc, cc], indexing="ij")
    q = (torch.stack([ox.reshape(-1), oy.reshape(-1), oz.reshape(-1)], 1) * .5 + .5)[None]
    w = (p * q + (1 - p) * (1 - q)).prod(-1)
    x = (w[..., None] * scene.values.double()[scene.feats.long()[v]]).sum(1)
    for li, lin in enumerate(field.layers):
        x = x @ lin.weight.double().t() + lin.bias.double()
        if li < len(field.layers) - 1:
            x = torch.relu(x)
    return x, p[:, 0]


@pytest.mark.parametrize("mlp", ["tc", "tc_fp8"])
def test_far_outside_samples_reevaluated_in_double_float(cuda, mlp):
    from nsvf_gb300 import ext, scenes, served
    from nsvf_gb300._lib import LIB
    enc, field, vs = _c2(cuda)
    rs, rd = scenes.frame_view(0, size=800)
    rs_t, rd_t = torch.from_numpy(rs).to(cuda), torch.from_numpy(rd).to(cuda)
    scene = served.SceneState(enc, field)
    out = served.render_frame(scene, rs_t, rd_t, mlp=mlp)
    ext.check_errors(cuda)
    b = next(iter(scene._frames.values()))
    n_far, ns, n_hit = out["n_far_outside"], out["n_samples"], out["n_hit_rays"]
    assert n_far > 100
    listed = torch.sort(b["outl"][:n_far])[0]
    # the standalone flag kernel lists the same samples
    lst = torch.empty(4 * n_far, dtype=torch.int64, device=cuda)
    cnt = torch.zeros(1, dtype=torch.int64, device=cuda)
    assert LIB.nsvf_flag_outliers(ns, None, b["vox"].data_ptr(), b["xyzd"].data_ptr(),
                                  scene.centers.size(0), scene.voxel_size,
                                  scene.centers.data_ptr(), lst.data_ptr(), cnt.data_ptr(),
                                  lst.numel(), None, ext.ctypes_stream(cuda)) == 0
    assert int(cnt) == n_far
    assert torch.equal(torch.sort(lst[:n_far])[0], listed)
    ref, p = _float64_field(scene, b["ro"], rd_t, b["depth"], b["vox"], b["pix"], b["offset"],
                            n_hit, listed, field)
    # every listed sample is far outside (float64 coordinates agree with the flag)
    assert ((p - 0.5).abs().max(-1)[0] > 0.999).all()
    got = b["field"][listed].double()
    scale = ref.abs().max(-1, keepdim=True)[0]
    err = (got - ref).abs()
    assert scale.max() > 10.0        # the extrapolated field is large there
    assert (err <= 2.0 ** -23 * ref.abs() + 1e-7 * scale).all(), float((err / scale).max())


def test_rays_with_large_extrapolated_colour_refined_in_fp32(cuda):
    """c4 (500,832 voxels, voxel 1/128), camera 0 at 800x800: the rays whose
    far-outside sample has a colour magnitude above served.REFINE_ABOVE get
    every other sample evaluated in FP32; those samples equal a torch FP32
    evaluation of the field (FP32 interpolation, nn.Linear layers) to FP32
    rounding, and the rest of the frame keeps its BF16 values."""
    from nsvf_gb300 import ext, scenes, served
    from nsvf_gb300.functional import trilinear_embed
    enc, field, vs = _c2(cuda, 1.0 / 128)
    rs, rd = scenes.frame_view(0, size=800)
    rs_t, rd_t = torch.from_numpy(rs).to(cuda), torch.from_numpy(rd).to(cuda)
    scene = served.SceneState(enc, field)
    out = served.render_frame(scene, rs_t, rd_t)
    ext.check_errors(cuda)
    b = next(iter(scene._frames.values()))
    n_ref = out["n_rays_refined_fp32"]
    assert n_ref > 10, out
    rows = torch.unique(b["outl"][b["outl_cap"]:b["outl_cap"] + n_ref])
    off = b["offset"]
    sel = torch.cat([torch.arange(int(off[r]), int(off[r + 1]), device=cuda) for r in rows.tolist()])
    far = torch.zeros(sel.numel(), dtype=torch.bool, device=cuda)
    far_set = b["outl"][:out["n_far_outside"]]
    far = torch.isin(sel, far_set)
    sel = sel[~far]
    emb = trilinear_embed(b["vox"][sel], b["xyzd"][sel, :3].contiguous(), scene.centers, scene.feats,
                          scene.values, scene.voxel_size)
    with torch.no_grad():
        ref = field.mlp(emb).float()
    got = b["field"][sel]
    scale = ref.abs().max(0)[0].clamp(min=1e-3)
    assert ((got - ref).abs() <= 1e-5 * scale).all(), float(((got - ref).abs() / scale).max())
