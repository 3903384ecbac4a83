"""The CPU oracle against the golden fixtures made by running the reference
(tests/golden/make_golden.py): this pins the oracle that the GPU tests use."""
import numpy as np
import pytest

from oracle import cpu


def test_aabb_raw(golden):
    g = golden
    R = g["ray_dir"].shape[0]
    rs = np.broadcast_to(g["ray_start"], (R, 3))[None]
    out = cpu.aabb_intersect(rs, g["ray_dir"][None], g["aabb_centers_shifted"][None],
                             float(g["voxel_size"]), 20)
    for got, key in zip(out, ["aabb_raw_idx", "aabb_raw_min", "aabb_raw_max"]):
        assert np.array_equal(got, g[key]), key


def test_svo_raw_and_sorted(golden):
    g = golden
    R = g["ray_dir"].shape[0]
    rs = np.broadcast_to(g["ray_start"], (R, 3))[None]
    out = cpu.svo_intersect(rs, g["ray_dir"][None], g["octree_centers"][None],
                            g["octree_children"][None], float(g["voxel_size"]), 20)
    for got, key in zip(out, ["svo_raw_idx", "svo_raw_min", "svo_raw_max"]):
        assert np.array_equal(got, g[key]), key
    idx, lo, hi = cpu.sort_hits(*out)
    # torch's sort is free to order ties differently; compare as (depth, id) sets
    assert np.array_equal(lo, g["svo_min_depth"])
    assert np.array_equal(np.sort(idx, -1), np.sort(g["svo_intersected_voxel_idx"], -1))
    assert np.array_equal((idx != -1).any(-1), g["svo_hits"])


def test_probs_steps(golden):
    g = golden
    probs, steps = cpu.probs_steps(g["svo_intersected_voxel_idx"][0], g["svo_min_depth"][0],
                                   g["svo_max_depth"][0], float(g["voxel_size"]) / 8)
    hit = g["svo_hits"][0]
    np.testing.assert_allclose(probs[hit], g["svo_probs"][0][hit], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(steps, g["svo_steps"][0], rtol=1e-6)


def _hit_rows(g):
    hit = g["svo_hits"][0]
    return (g["svo_intersected_voxel_idx"][0][hit], g["svo_min_depth"][0][hit],
            g["svo_max_depth"][0][hit], g["svo_probs"][0][hit], g["svo_steps"][0][hit])


def test_inverse_cdf_deterministic(golden):
    g = golden
    I, lo, hi, pr, st = _hit_rows(g)
    N, P = I.shape
    M = int(np.ceil(st).max()) + P
    noise = np.full((N, M), 0.5, np.float32)
    si, sd, ss = cpu.inverse_cdf_op(I, lo, hi, pr, st, noise)
    # the encoder's post-processing (fairnr/modules/encoder.py:547-549)
    ss = np.maximum(ss, 0)
    sd = np.where(si == -1, np.float32(10000.0), sd)
    ss = np.where(si == -1, np.float32(0.0), ss)
    assert np.array_equal(si, g["svo_det_sampled_point_voxel_idx"])
    assert np.array_equal(sd, g["svo_det_sampled_point_depth"])
    assert np.array_equal(ss, g["svo_det_sampled_point_distance"])


def test_inverse_cdf_recorded_noise(golden):
    g = golden
    I, lo, hi, pr, st = _hit_rows(g)
    si, sd, ss = cpu.inverse_cdf_op(I, lo, hi, pr, st, g["svo_noise"])
    ss = np.maximum(ss, 0)
    sd = np.where(si == -1, np.float32(10000.0), sd)
    ss = np.where(si == -1, np.float32(0.0), ss)
    assert np.array_equal(si, g["svo_rand_sampled_point_voxel_idx"])
    assert np.array_equal(sd, g["svo_rand_sampled_point_depth"])
    assert np.array_equal(ss, g["svo_rand_sampled_point_distance"])


def _samples_xyz(g):
    hit = g["svo_hits"][0]
    rd = g["ray_dir"][hit].astype(np.float32)
    d = g["svo_det_sampled_point_depth"]
    xyz = g["ray_start"][None, None, :] + rd[:, None, :] * d[..., None]
    mask = g["svo_det_sampled_point_voxel_idx"] != -1
    return xyz.astype(np.float32), mask


def test_trilinear_embedding(golden):
    g = golden
    xyz, mask = _samples_xyz(g)
    vidx = g["svo_det_sampled_point_voxel_idx"][mask]
    emb = cpu.trilinear_embed(xyz[mask], vidx, g["svo_centers_shifted"], g["feats"], g["embed"],
                              float(g["voxel_size"]))
    n = g["svo_det_emb"].shape[0]
    np.testing.assert_allclose(emb[:n], g["svo_det_emb"], rtol=1e-4, atol=1e-5)


def test_render(golden):
    g = golden
    xyz, mask = _samples_xyz(g)
    vidx = g["svo_det_sampled_point_voxel_idx"]
    emb = cpu.trilinear_embed(xyz[mask], vidx[mask], g["svo_centers_shifted"], g["feats"],
                              g["embed"], float(g["voxel_size"]))
    sig, rgb = cpu.mlp_forward(emb, [(g["W%d" % i], g["b%d" % i]) for i in range(5)])
    S = np.zeros(mask.shape)
    C = np.zeros(mask.shape + (3,))
    S[mask], C[mask] = sig, rgb
    out = cpu.composite(S, C, g["svo_det_sampled_point_depth"].astype(np.float64),
                        g["svo_det_sampled_point_distance"].astype(np.float64), mask)
    np.testing.assert_allclose(out["colors"], g["render_colors"], atol=2e-4)
    np.testing.assert_allclose(out["missed"], g["render_missed"], atol=2e-4)
    np.testing.assert_allclose(out["depths"], g["render_depths"], rtol=1e-4, atol=2e-3)
    np.testing.assert_allclose(out["probs"], g["render_probs"], atol=2e-4)


def test_octree_builder(golden):
    import torch
    from nsvf_gb300 import geometry
    g = golden
    pts = torch.from_numpy(g["points"])
    coords, residual = geometry.discretize_points(pts, float(g["voxel_size"]) / 2)
    ranges = coords.max(0)[0] - coords.min(0)[0]
    depth = int(torch.log2(ranges.max().float()).ceil_().long() - 1)
    center = ((coords.max(0)[0] + coords.min(0)[0]) / 2).numpy()
    cen, chi = cpu.build_octree(center, coords.numpy(), depth)
    assert np.array_equal(chi, g["octree_children"])
    cenf = cen.astype(np.float32) * np.float32(float(g["voxel_size"]) / 2) + residual.numpy()
    assert np.array_equal(cenf.astype(np.float32), g["octree_centers"])
