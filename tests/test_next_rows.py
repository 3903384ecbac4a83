"""The steps either side of the rendering path, against fixtures made by the
reference's own code (tests/golden/make_golden_next.py):

* ray generation in the reference's camera convention: get_uv and
  get_ray_direction (torch, CPU) and the nsvf_camera_rays kernel (GPU);
* voxel splitting with embedding re-interpolation (SparseVoxelEncoder.
  splitting), on the CPU;
* the renderer's early termination (raymarching_tolerance: the column-chunk
  loop stops evaluating rays whose accumulated free energy passed -log tol),
  on the GPU: the same field evaluations ('ae') and the same image.

Tolerances: ray directions 2e-6 (unit vectors; the reference's 4x4 matmul
and norm sum in a different order); splitting: centres and corner ids exact,
embeddings 1e-6; early-terminated render 2e-4 (the FP32 compositing kernels
against the reference's torch cumsum, as for the full render)."""
import argparse
import os
import tempfile

import numpy as np
import pytest
import torch


def _encoder(golden, dev):
    from nsvf_gb300.encoder import SparseVoxelEncoder
    g = golden
    path = tempfile.mktemp(suffix=".txt")
    np.savetxt(path, np.array([[-1, -1, -1, 1, 1, 1, float(g["voxel_size"])]]))
    args = argparse.Namespace(voxel_path=None, initial_boundingbox=path,
                              voxel_size=float(g["voxel_size"]), max_hits=20,
                              raymarching_stepsize_ratio=0.125, voxel_embed_dim=32,
                              use_octree=True, deterministic_step=True)
    enc = SparseVoxelEncoder(args)
    os.unlink(path)
    enc.keep.copy_(torch.from_numpy(g["keep"]))
    enc.values.weight.data.copy_(torch.from_numpy(g["embed"][: enc.values.weight.shape[0]]))
    return enc.to(dev).eval()


def test_get_uv_and_ray_direction_match_reference(golden_next):
    from nsvf_gb300 import geometry
    g = golden_next
    H, W, h, w = [int(x) for x in g["rays_hw"]]
    uv, ratio = geometry.get_uv(H, W, h, w)
    assert np.array_equal(uv.reshape(2, -1), g["rays_uv"])
    assert ratio == [H / h, W / w]
    inv_RT = torch.from_numpy(g["rays_inv_RT"])
    fx, fy, cx, cy = [float(x) for x in g["rays_intrinsics"]]
    K = torch.eye(4)
    K[0, 0], K[1, 1], K[0, 2], K[1, 2] = fx, fy, cx, cy
    d = geometry.get_ray_direction(inv_RT[:3, 3], torch.from_numpy(uv.reshape(2, -1)), K, inv_RT)
    np.testing.assert_allclose(d.t().numpy(), g["rays_dir"], atol=2e-6)


def test_splitting_matches_reference(golden, golden_next):
    g, n = golden, golden_next
    enc = _encoder(g, "cpu")
    enc.splitting()
    assert np.array_equal(enc.points.numpy(), n["split_points"])
    assert np.array_equal(enc.feats.numpy(), n["split_feats"])
    assert int(enc.num_keys) == int(n["split_num_keys"])
    assert np.array_equal(enc.keep.numpy(), n["split_keep"])
    np.testing.assert_allclose(enc.values.weight.detach().numpy(), n["split_values"], atol=1e-6)


@pytest.mark.gpu
def test_camera_rays_kernel_matches_reference(golden_next, cuda):
    from nsvf_gb300 import ext
    g = golden_next
    H, W, h, w = [int(x) for x in g["rays_hw"]]
    ro, rd = ext.camera_rays(g["rays_intrinsics"], g["rays_inv_RT"], H, W, h, w, device=cuda)
    np.testing.assert_allclose(rd.cpu().numpy(), g["rays_dir"], atol=2e-6)
    assert np.array_equal(ro.cpu().numpy(), np.broadcast_to(g["rays_start"], ro.shape))
    # a chunk of the same frame: pixels 100..299
    ro2, rd2 = ext.camera_rays(g["rays_intrinsics"], g["rays_inv_RT"], H, W, h, w, first=100, n=200,
                               device=cuda)
    assert torch.equal(rd2, rd[100:300])


@pytest.mark.gpu
@pytest.mark.parametrize("tol", [0.01, 0.5])
def test_early_termination_matches_reference(golden, golden_next, cuda, tol):
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.renderer import VolumeRenderer
    g, n = golden, golden_next
    enc = _encoder(g, cuda)
    st = enc.precompute(id=None)
    field = StandInField(weights=[(torch.from_numpy(g["W%d" % i]), torch.from_numpy(g["b%d" % i]))
                                  for i in range(5)]).to(cuda).eval()
    hit = g["svo_hits"][0]
    N = int(hit.sum())
    rs = torch.from_numpy(g["ray_start"]).to(cuda).reshape(1, 3).expand(N, 3)
    rd = torch.from_numpy(g["ray_dir"][hit]).to(cuda)
    samples = {k: torch.from_numpy(g["svo_det_%s" % k]).to(cuda)
               for k in ["sampled_point_depth", "sampled_point_distance", "sampled_point_voxel_idx"]}
    ren = VolumeRenderer(argparse.Namespace(chunk_size=1, raymarching_tolerance=tol)).eval()
    with torch.no_grad():
        out = ren(enc, field, rs, rd, samples, st)
    tag = "es%g" % tol
    assert int(out["ae"]) == int(n["%s_ae" % tag])
    for k in ["colors", "depths", "missed"]:
        np.testing.assert_allclose(out[k].cpu().numpy(), n["%s_%s" % (tag, k)], atol=2e-4)
    np.testing.assert_allclose(out["probs"].cpu().numpy(), n["%s_probs" % tag], atol=2e-4)
    # and it does stop early: fewer evaluations than valid samples
    assert int(out["ae"]) < int((g["svo_det_sampled_point_voxel_idx"] != -1).sum())


def _tri_golden_faces(n):
    verts, faces = n["tri_verts"], n["tri_faces"]
    return verts[faces].reshape(1, -1, 9).astype(np.float32)


def test_triangle_oracle_matches_reference(golden_next):
    """The mesh encoder's ray-triangle op: the C oracle against the
    reference's own triangle_ray_intersect output, bit for bit."""
    from oracle import cpu
    n = golden_next
    idx, depth, uv = cpu.triangle_intersect(n["tri_ray_start"], n["tri_ray_dir"],
                                            _tri_golden_faces(n), 0.05, 0.01, 8)
    assert np.array_equal(idx, n["tri_inds"])
    assert np.array_equal(depth.reshape(n["tri_depth"].shape), n["tri_depth"])
    assert np.array_equal(uv, n["tri_uv"])
    assert (idx != -1).sum() > 200


@pytest.mark.gpu
def test_triangle_ray_intersect_matches_reference(golden_next, cuda):
    from nsvf_gb300 import clib
    n = golden_next
    out = clib.triangle_ray_intersect(0.05, 0.01, 8, torch.from_numpy(n["tri_verts"]).to(cuda),
                                      torch.from_numpy(n["tri_faces"]).to(cuda),
                                      torch.from_numpy(n["tri_ray_start"]).to(cuda),
                                      torch.from_numpy(n["tri_ray_dir"]).to(cuda))
    for got, key in zip(out, ["tri_inds", "tri_depth", "tri_uv"]):
        assert np.array_equal(got.cpu().numpy(), n[key]), key


@pytest.mark.gpu
@pytest.mark.parametrize("n_faces,n_max,blur,shared", [(37, 4, 0.0, True), (700, 16, 0.05, False),
                                                       (1500, 8, 0.0, True)])
def test_triangle_kernel_matches_oracle(cuda, n_faces, n_max, blur, shared):
    """Random triangle soups (more faces than one shared-memory tile in the
    larger cases), faces shared by both ray rows or one set per row."""
    from nsvf_gb300 import ext
    from oracle import cpu
    rng = np.random.RandomState(n_faces)
    b, m = 2, 700
    nb = 1 if shared else b
    faces = rng.uniform(-1, 1, size=(nb, n_faces, 9)).astype(np.float32)
    o = (rng.normal(size=(b, m, 3)) * 3).astype(np.float32)
    d = (-o + rng.normal(scale=0.5, size=(b, m, 3))).astype(np.float32)
    d = (d / np.linalg.norm(d, axis=-1, keepdims=True)).astype(np.float32)
    got = ext.triangle_intersect(torch.from_numpy(o).to(cuda), torch.from_numpy(d).to(cuda),
                                 torch.from_numpy(faces).to(cuda), 0.03, blur, n_max)
    ref = cpu.triangle_intersect(o, d, np.broadcast_to(faces, (b, n_faces, 9)), 0.03, blur, n_max)
    for a, r in zip(got, ref):
        assert np.array_equal(a.cpu().numpy(), r)
    assert (ref[0] != -1).sum() > 500


@pytest.mark.gpu
def test_reference_radiance_field_renders_like_reference(golden, golden_next, cuda):
    """A checkpoint of the reference's RaidanceField (state dict from the
    fixture) loads into nsvf_gb300.field.RaidanceField and renders the same
    samples through the drop-in encoder and renderer as the reference did."""
    from nsvf_gb300.field import RaidanceField
    from nsvf_gb300.renderer import VolumeRenderer
    g, n = golden, golden_next
    enc = _encoder(g, cuda)
    st = enc.precompute(id=None)
    args = argparse.Namespace(inputs_to_density="emb:6:32", inputs_to_texture="feat:0:64, ray:4",
                              feature_embed_dim=64, density_embed_dim=32, texture_embed_dim=64,
                              feature_layers=1, texture_layers=2, background_stop_gradient=False)
    field = RaidanceField(args)
    state = {k[len("rf_state_"):]: torch.from_numpy(n[k]) for k in n if k.startswith("rf_state_")}
    field.load_state_dict(state, strict=True)
    field = field.to(cuda).eval()
    hit = g["svo_hits"][0]
    N = int(hit.sum())
    rs = torch.from_numpy(g["ray_start"]).to(cuda).reshape(1, 3).expand(N, 3)
    rd = torch.from_numpy(g["ray_dir"][hit]).to(cuda)
    samples = {k: torch.from_numpy(g["svo_det_%s" % k]).to(cuda)
               for k in ["sampled_point_depth", "sampled_point_distance", "sampled_point_voxel_idx"]}
    ren = VolumeRenderer(argparse.Namespace(chunk_size=64)).eval()
    with torch.no_grad():
        out = ren(enc, field, rs, rd, samples, st)
    for k in ["colors", "depths", "missed"]:
        np.testing.assert_allclose(out[k].cpu().numpy(), n["rf_%s" % k], atol=2e-4)
    assert float(n["rf_missed"].min()) < 0.1          # an opaque enough field to test compositing


@pytest.mark.gpu
def test_reference_radiance_field_in_served_chain(golden, golden_next, cuda):
    """The same checkpointed RaidanceField in the served chain
    (served.SceneState + render_frame, mlp="field": the field's FP32 torch
    modules on the compacted samples) renders the frame of the drop-in
    module path."""
    from nsvf_gb300.field import RaidanceField
    from nsvf_gb300.renderer import VolumeRenderer, render_rays
    from nsvf_gb300.served import SceneState, render_frame
    g, n = golden, golden_next
    enc = _encoder(g, cuda)
    args = argparse.Namespace(inputs_to_density="emb:6:32", inputs_to_texture="feat:0:64, ray:4",
                              feature_embed_dim=64, density_embed_dim=32, texture_embed_dim=64,
                              feature_layers=1, texture_layers=2, background_stop_gradient=False)
    field = RaidanceField(args)
    state = {k[len("rf_state_"):]: torch.from_numpy(n[k]) for k in n if k.startswith("rf_state_")}
    field.load_state_dict(state, strict=True)
    field = field.to(cuda).eval()
    rs = torch.from_numpy(g["ray_start"]).to(cuda).reshape(3)
    rd = torch.from_numpy(g["ray_dir"]).to(cuda)
    ren = VolumeRenderer(argparse.Namespace(chunk_size=64)).eval()
    with torch.no_grad():
        ref = render_rays(enc, field, ren, rs.reshape(1, 1, 1, 3), rd.reshape(1, 1, -1, 3))
    scene = SceneState(enc, field)
    assert scene.mlp is None                   # not the 4 x 128 tensor-core field
    out = render_frame(scene, rs, rd, kahan=False)
    assert out["n_samples"] > 1000
    for k in ["colors", "depths", "missed"]:
        np.testing.assert_allclose(out[k].cpu().numpy(), ref[k].reshape(out[k].shape).cpu().numpy(),
                                   atol=2e-4, err_msg=k)
    assert float(out["missed"].min()) < 0.1


@pytest.mark.gpu
def test_splitting_on_gpu_then_render(golden, golden_next, cuda):
    """Splitting on the device gives the reference's split voxels, corner
    table and keep mask (the embeddings re-interpolated to 1e-6); the split
    scene (voxel size halved, max_hits x 1.5, as the reference's model does
    after splitting: fairnr/models/nsvf.py) then rebuilds its octree and
    renders through the served chain the frame of the drop-in path.
    (fairnr/models/nsvf.py:148-155: splitting, voxel size x 0.5, max_hits x
    1.5, runtime caches cleared.)"""
    from nsvf_gb300 import scenes
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.renderer import VolumeRenderer, render_rays
    from nsvf_gb300.served import SceneState, render_frame
    g, n = golden, golden_next
    enc = _encoder(g, cuda)
    enc.splitting()
    assert np.array_equal(enc.points.cpu().numpy(), n["split_points"])
    assert np.array_equal(enc.feats.cpu().numpy(), n["split_feats"])
    assert int(enc.num_keys) == int(n["split_num_keys"])
    assert np.array_equal(enc.keep.cpu().numpy(), n["split_keep"])
    np.testing.assert_allclose(enc.values.weight.detach().cpu().numpy(), n["split_values"],
                               atol=1e-6)
    enc.voxel_size *= .5
    enc.max_hits *= 1.5
    enc.clean_runtime_caches()
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=2, sigma_scale=30.0,
                                                             sigma_bias=0.5)).to(cuda).eval()
    rs = torch.from_numpy(g["ray_start"]).to(cuda).reshape(3)
    rd = torch.from_numpy(g["ray_dir"]).to(cuda)
    ren = VolumeRenderer(argparse.Namespace(chunk_size=64)).eval()
    with torch.no_grad():
        ref = render_rays(enc, field, ren, rs.reshape(1, 1, 1, 3), rd.reshape(1, 1, -1, 3))
    out = render_frame(SceneState(enc, field), rs, rd, mlp="fp32", kahan=False, exact=False)
    assert out["n_samples"] > 1000
    for k in ["colors", "missed"]:
        np.testing.assert_allclose(out[k].cpu().numpy(), ref[k].reshape(out[k].shape).cpu().numpy(),
                                   atol=2e-5, err_msg=k)
