"""Hierarchical resampling (renderer.prepare_hierarchical_sampling and
render_rays(hierarchical=True)) against the reference's own
prepare_hierarchical_sampling, fine inverse-CDF samples and fine render
(golden_hier.npz, tests/golden/make_golden_hier.py) on the 147-voxel scene:
NeRF's fixed 64 fine samples and NSVF's 2x the coarse count.

The fine-pass inputs match bit for bit except the normalised probabilities,
whose per-ray sum the reference takes in torch's pairwise order (~1e-6
relative: the sequential sum adds the 1e-5 padding terms one by one); given the
reference's inputs the fine samples match bit for bit and the fine render to
FP32 rounding."""
import argparse
import os
import tempfile

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SETTINGS = [("nerf64", dict(fixed_fine_num_samples=64)),
            ("nsvf2", dict(fine_num_sample_ratio=2.0))]


def _golden_encoder(g, dev):
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.renderer import VolumeRenderer
    path = tempfile.mktemp(suffix=".txt")
    np.savetxt(path, np.array([[-1, -1, -1, 1, 1, 1, float(g["voxel_size"])]]))
    args = argparse.Namespace(voxel_path=None, initial_boundingbox=path,
                              voxel_size=float(g["voxel_size"]), max_hits=20,
                              raymarching_stepsize_ratio=0.125, voxel_embed_dim=32,
                              use_octree=True, deterministic_step=True, chunk_size=64)
    enc = SparseVoxelEncoder(args)
    os.unlink(path)
    enc.keep.copy_(torch.from_numpy(g["keep"]))
    enc.values.weight.data.copy_(torch.from_numpy(g["embed"][: enc.values.weight.shape[0]]))
    field = StandInField(weights=[(torch.from_numpy(g["W%d" % i]), torch.from_numpy(g["b%d" % i]))
                                  for i in range(5)])
    return enc.to(dev).eval(), field.to(dev).eval(), VolumeRenderer(args).eval()


@pytest.mark.parametrize("tag,kw", SETTINGS)
def test_prepare_hierarchical_matches_reference(golden, golden_hier, cuda, tag, kw):
    from nsvf_gb300.renderer import prepare_hierarchical_sampling
    g, gh = golden, golden_hier
    t = lambda k: torch.from_numpy(g[k]).to(cuda)
    samples = {k: t("svo_det_%s" % k) for k in
               ["sampled_point_depth", "sampled_point_distance", "sampled_point_voxel_idx"]}
    io = prepare_hierarchical_sampling({}, samples, {"probs": t("render_probs")}, **kw)
    for k in ["min_depth", "max_depth", "intersected_voxel_idx", "steps"]:
        assert np.array_equal(io[k].cpu().numpy(), gh["%s_%s" % (tag, k)]), k
    # a sequential sum adds the ~1e-5 padding terms onto ~1 one by one; torch's
    # pairwise sum keeps them apart: ~1e-6 relative
    np.testing.assert_allclose(io["probs"].cpu().numpy(), gh["%s_probs" % tag], rtol=5e-6, atol=0)


@pytest.mark.parametrize("tag,kw", SETTINGS)
def test_fine_samples_and_render_match_reference(golden, golden_hier, cuda, tag, kw):
    g, gh = golden, golden_hier
    enc, field, ren = _golden_encoder(g, cuda)
    io = {k: torch.from_numpy(gh["%s_%s" % (tag, k)]).to(cuda)
          for k in ["min_depth", "max_depth", "intersected_voxel_idx", "probs", "steps"]}
    fine = enc.ray_sample(io)
    for k, v in fine.items():
        assert np.array_equal(v.cpu().numpy(), gh["%s_fine_%s" % (tag, k)]), k
    hit = g["svo_hits"][0]
    rs = torch.from_numpy(g["ray_start"]).to(cuda).reshape(1, 3).expand(int(hit.sum()), 3)
    rd = torch.from_numpy(g["ray_dir"][hit]).to(cuda)
    with torch.no_grad():
        res = ren(enc, field.forward, rs, rd, dict(fine), enc.precompute(id=None))
    for k in ["colors", "depths", "missed"]:
        np.testing.assert_allclose(res[k].cpu().numpy(), gh["%s_render_%s" % (tag, k)],
                                   atol=2e-5, rtol=1e-5)


def test_render_rays_hierarchical(golden, golden_hier, cuda):
    """render_rays(hierarchical=True) end to end (coarse pass, resampling,
    fine pass, background fill) against the reference's fine render: the
    coarse probabilities differ from the reference's by FP32 rounding, which
    can move a fine sample, so colours agree to 1e-3."""
    from nsvf_gb300.renderer import render_rays
    g, gh = golden, golden_hier
    enc, field, ren = _golden_encoder(g, cuda)
    hit = g["svo_hits"][0]
    rs = torch.from_numpy(g["ray_start"]).to(cuda).reshape(1, 1, 1, 3)
    rd = torch.from_numpy(g["ray_dir"]).to(cuda).reshape(1, 1, -1, 3)
    with torch.no_grad():
        out = render_rays(enc, field, ren, rs, rd, hierarchical=True, fixed_fine_num_samples=64)
    col = out["colors"].reshape(-1, 3)[torch.from_numpy(hit).to(cuda)].cpu().numpy()
    ref = gh["nerf64_render_colors"] + gh["nerf64_render_missed"][:, None]
    np.testing.assert_allclose(col, ref, atol=1e-3)
    assert "coarse" in out and out["coarse"]["colors"].shape == out["colors"].shape
