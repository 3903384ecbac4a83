"""Precision: the float64 GPU validation render against the CPU oracle, and
the error budget of the served BF16 and drop-in FP32 frames against it
(workloads' field: max RGB error <= 2e-3 served, <= 1e-4 FP32), on a small
frame and over every pixel of the full 800x800 c2 and c4 frames."""
import argparse

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _scene(dev, voxel, std, ss, sb, H):
    from nsvf_gb300 import scenes
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.renderer import VolumeRenderer
    p, vs = scenes.scene_small() if voxel == 0.25 else scenes.scene_shell(voxel)
    args = argparse.Namespace(voxel_size=vs, max_hits=H, raymarching_stepsize_ratio=0.125,
                              voxel_embed_dim=32, use_octree=True, deterministic_step=True,
                              chunk_size=64)
    enc = SparseVoxelEncoder(args, points=p)
    with torch.no_grad():
        enc.values.weight.copy_(scenes.voxel_embeddings(enc.values.weight.shape[0], 32, std, seed=1))
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=2, sigma_scale=ss, sigma_bias=sb))
    return enc.to(dev).eval(), field.to(dev).eval(), VolumeRenderer(args).eval(), vs


def test_fp64_render_matches_cpu_oracle(cuda):
    from nsvf_gb300 import scenes
    from nsvf_gb300.precision import fp64_render
    from oracle import cpu
    enc, field, ren, vs = _scene(cuda, 0.25, 1.0, 60.0, 0.5, 20)
    rs, rd = scenes.small_view(0)
    col, dep, hits, _, _ = fp64_render(enc, field, torch.from_numpy(rs).to(cuda), torch.from_numpy(rd).to(cuda))
    st = enc.precompute(id=None)
    cen, chi = st['voxel_octree_center_xyz'].cpu().numpy(), st['voxel_octree_children_idx'].cpu().numpy()
    R = rd.shape[0]
    idx, lo, hi = cpu.sort_hits(*cpu.svo_intersect(np.broadcast_to(rs, (R, 3))[None], rd[None],
                                                   cen[None], chi[None], vs, 20))
    idx, lo, hi = idx[0], lo[0], hi[0]
    hit = (idx != -1).any(-1)
    assert np.array_equal(hit, hits.cpu().numpy())
    pr, stp = cpu.probs_steps(idx[hit], lo[hit], hi[hit], vs / 8)
    N = int(hit.sum())
    M = int(np.ceil(stp).max()) + 20
    si, sd, ss = cpu.inverse_cdf_op(idx[hit], lo[hit], hi[hit], pr, stp, np.full((N, M), 0.5, np.float32))
    ss = np.maximum(ss, 0)
    mask = si != -1
    xyz = rs[None, None].astype(np.float64) + rd[hit][:, None].astype(np.float64) * sd[..., None]
    emb = cpu.trilinear_embed(xyz[mask], si[mask], st['voxel_center_xyz'].cpu().numpy(),
                              st['voxel_vertex_idx'].cpu().numpy(),
                              st['voxel_vertex_emb'].detach().cpu().numpy(), vs)
    W = [(l.weight.detach().cpu().numpy(), l.bias.detach().cpu().numpy()) for l in field.layers]
    sig, rgb = cpu.mlp_forward(emb, W)
    S = np.zeros(mask.shape)
    C = np.zeros(mask.shape + (3,))
    S[mask], C[mask] = sig, rgb
    o = cpu.composite(S, C, sd.astype(np.float64), ss.astype(np.float64), mask)
    ref = np.ones((R, 3))
    ref[hit] = o["colors"] + o["missed"][:, None]
    np.testing.assert_allclose(col.cpu().numpy(), ref, atol=1e-9)


def test_error_budget_against_fp64(cuda):
    from nsvf_gb300 import scenes
    from nsvf_gb300.precision import report
    enc, field, ren, vs = _scene(cuda, 1.0 / 32, 0.01, 1.0, 0.0, 64)
    rs, rd = scenes.frame_view(3, size=160)
    rep = report(enc, field, ren, torch.from_numpy(rs).to(cuda), torch.from_numpy(rd).to(cuda))
    assert rep["hit_pixels"] > 1000
    assert rep["served_bf16"]["max_rgb_err"] <= 2e-3, rep
    print("precision report:", rep)
    # the FP8 option: E4M3 hidden layers cost about an order of magnitude
    assert rep["served_fp8"]["max_rgb_err"] <= 5e-2, rep
    assert rep["plain_fp32"]["max_rgb_err"] <= 1e-4, rep


@pytest.mark.parametrize("voxel,cam", [(1.0 / 64, 0), (1.0 / 128, 0), (1.0 / 64, 91)])
def test_full_frame_error_bar_every_pixel(cuda, voxel, cam):
    """c2 (125,476 voxels, voxel 1/64) and c4 (500,832 voxels, voxel 1/128):
    camera 0 at 800x800, and c2's camera 91 (the largest error of seven c2
    cameras measured: 1.0e-3). The served BF16 frame and the served chain
    with the FP32 field meet the 2e-3 max RGB error bar against the float64
    render on every pixel, including the ~0.1-0.2 % of hit pixels with a
    sample far outside its voxel (evaluated again in double-float)."""
    from nsvf_gb300 import scenes
    from nsvf_gb300.precision import report
    enc, field, ren, vs = _scene(cuda, voxel, 0.01, 1.0, 0.0, 64)
    rs, rd = scenes.frame_view(cam, size=800)
    rep = report(enc, field, ren, torch.from_numpy(rs).to(cuda), torch.from_numpy(rd).to(cuda))
    print("precision report:", rep)
    assert rep["hit_pixels"] > 100000
    assert rep["samples_outside_their_voxel"] > 500
    assert rep["samples_reevaluated_in_double_float"] >= rep["samples_outside_their_voxel"] - 2
    assert rep["served_bf16"]["max_rgb_err"] <= 2e-3, rep["served_bf16"]
    assert rep["served_fp32"]["max_rgb_err"] <= 2e-3, rep["served_fp32"]
    assert rep["served_bf16"]["max_depth_err_hit_pixels"] <= 1e-2, rep["served_bf16"]
