"""The rendering side on the GPU: trilinear interpolation and compositing
kernels (forward and hand-written backward) against float64 torch references
of the same formulas, and the drop-in encoder/renderer end to end against
the golden render made by the reference's own modules.

Tolerances: FP32 kernels vs float64 references: 1e-5 absolute on
embeddings, 1e-5 on compositing outputs (their summation order differs from
torch's); end-to-end colours vs the reference's FP32 render: 2e-4."""
import argparse

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _trilinear_ref(idx, xyz, centers, feats, values, vs):
    """float64 torch restatement of fairnr/modules/encoder.py:584-590."""
    c = centers.double()[idx]
    p = ((xyz.double() - c) / vs + .5).unsqueeze(1)
    cc = torch.tensor([-1.0, 1.0], dtype=torch.float64, device=xyz.device)
    ox, oy, oz = torch.meshgrid([cc, cc, cc], indexing="ij")
    q = (torch.stack([ox.reshape(-1), oy.reshape(-1), oz.reshape(-1)], 1) * .5 + .5).unsqueeze(0)
    w = (p * q + (1 - p) * (1 - q)).prod(-1, keepdim=True)
    v = values.double()[feats[idx]]
    return (w * v).sum(1)


def test_trilinear_forward_backward(golden, cuda):
    from nsvf_gb300.functional import trilinear_embed
    g = golden
    hit = g["svo_hits"][0]
    rd = g["ray_dir"][hit]
    d = g["svo_det_sampled_point_depth"]
    mask = g["svo_det_sampled_point_voxel_idx"] != -1
    xyz = (g["ray_start"][None, None] + rd[:, None] * d[..., None]).astype(np.float32)[mask]
    idx = _t(g["svo_det_sampled_point_voxel_idx"][mask].astype(np.int64), cuda)
    xyz = _t(xyz, cuda).requires_grad_(True)
    centers = _t(g["svo_centers_shifted"], cuda)
    feats = _t(g["feats"], cuda)
    values = _t(g["embed"], cuda).requires_grad_(True)
    vs = float(g["voxel_size"])
    emb = trilinear_embed(idx, xyz, centers, feats, values, vs)
    n = g["svo_det_emb"].shape[0]
    np.testing.assert_allclose(emb[:n].detach().cpu().numpy(), g["svo_det_emb"], atol=1e-5)
    # backward against autograd of the float64 restatement
    x64 = xyz.detach().double().requires_grad_(True)
    v64 = values.detach().double().requires_grad_(True)
    ref = _trilinear_ref(idx, x64, centers, feats, v64, vs)
    np.testing.assert_allclose(emb.detach().cpu().numpy(), ref.detach().cpu().numpy(), atol=1e-5)
    gout = torch.randn_like(emb)
    (emb * gout).sum().backward()
    (ref * gout.double()).sum().backward()
    np.testing.assert_allclose(values.grad.cpu().numpy(), v64.grad.cpu().numpy(), atol=1e-4)
    np.testing.assert_allclose(xyz.grad.cpu().numpy(), x64.grad.cpu().numpy(), rtol=1e-4, atol=1e-3)


def _composite_ref(fe, tex, t):
    sh = torch.cat([fe.new_zeros(fe.size(0), 1), fe[:, :-1]], 1)
    a = 1 - torch.exp(-fe)
    b = torch.exp(-torch.cumsum(sh, 1))
    p = a * b
    return p, (t * p).sum(-1), 1 - p.sum(-1), (tex * p.unsqueeze(-1)).sum(1)


@pytest.mark.parametrize("kahan", [False, True])
@pytest.mark.parametrize("R,M", [(7, 5), (300, 97), (64, 600)])
def test_composite_forward_backward(cuda, R, M, kahan):
    from nsvf_gb300.functional import composite
    gen = torch.Generator(device="cpu").manual_seed(R * M)
    fe = (torch.rand(R, M, generator=gen) * 0.2).to(cuda)
    fe[:, M // 2:] *= (torch.rand(R, 1, generator=gen) > 0.5).float().to(cuda)   # ragged tails
    tex = torch.randn(R, M, 3, generator=gen).to(cuda)
    t = torch.sort(torch.rand(R, M, generator=gen) * 4, 1)[0].to(cuda)
    fe.requires_grad_(True)
    tex.requires_grad_(True)
    out = composite(fe, tex, t, kahan)
    fe64 = fe.detach().double().requires_grad_(True)
    tex64 = tex.detach().double().requires_grad_(True)
    ref = _composite_ref(fe64, tex64, t.double())
    for a, b in zip(out, ref):
        np.testing.assert_allclose(a.detach().cpu().numpy(), b.detach().cpu().numpy(), atol=1e-5,
                                   rtol=1e-5)
    gs = [torch.randn_like(o) for o in out]
    sum((o * g).sum() for o, g in zip(out, gs)).backward()
    sum((o * g.double()).sum() for o, g in zip(ref, gs)).backward()
    np.testing.assert_allclose(fe.grad.cpu().numpy(), fe64.grad.cpu().numpy(), atol=2e-4, rtol=1e-4)
    np.testing.assert_allclose(tex.grad.cpu().numpy(), tex64.grad.cpu().numpy(), atol=1e-5)


def _encoder(golden, dev, use_octree=True):
    import tempfile, os
    from nsvf_gb300.encoder import SparseVoxelEncoder
    g = golden
    path = tempfile.mktemp(suffix=".txt")
    np.savetxt(path, np.array([[-1, -1, -1, 1, 1, 1, float(g["voxel_size"])]]))
    args = argparse.Namespace(voxel_path=None, initial_boundingbox=path,
                              voxel_size=float(g["voxel_size"]), max_hits=20,
                              raymarching_stepsize_ratio=0.125, voxel_embed_dim=32,
                              use_octree=use_octree, deterministic_step=True)
    enc = SparseVoxelEncoder(args)
    os.unlink(path)
    enc.keep.copy_(torch.from_numpy(g["keep"]))
    enc.values.weight.data.copy_(torch.from_numpy(g["embed"][: enc.values.weight.shape[0]]))
    return enc.to(dev).eval()


def test_encoder_intersect_matches_golden(golden, cuda):
    g = golden
    for use_octree, tag in [(True, "svo"), (False, "aabb")]:
        enc = _encoder(g, cuda, use_octree)
        st = enc.precompute(id=None)
        rd = _t(g["ray_dir"], cuda).reshape(1, 1, -1, 3)
        rs = _t(g["ray_start"], cuda).reshape(1, 1, 1, 3)
        _, _, out, hits = enc.ray_intersect(rs, rd, {k: (v.unsqueeze(0) if v is not None else None)
                                                      for k, v in st.items()})
        assert np.array_equal(out["min_depth"].cpu().numpy(), g["%s_min_depth" % tag])
        assert np.array_equal(out["max_depth"].cpu().numpy(), g["%s_max_depth" % tag])
        assert np.array_equal(hits.cpu().numpy(), g["%s_hits" % tag])
        a = out["intersected_voxel_idx"].cpu().numpy()
        assert np.array_equal(np.sort(a, -1), np.sort(g["%s_intersected_voxel_idx" % tag], -1))


def test_render_rays_matches_golden(golden, cuda):
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.renderer import VolumeRenderer, render_rays
    g = golden
    enc = _encoder(g, cuda, True)
    field = StandInField(weights=[(torch.from_numpy(g["W%d" % i]), torch.from_numpy(g["b%d" % i]))
                                  for i in range(5)]).to(cuda).eval()
    ren = VolumeRenderer(argparse.Namespace(chunk_size=64)).eval()
    rd = _t(g["ray_dir"], cuda).reshape(1, 1, -1, 3)
    rs = _t(g["ray_start"], cuda).reshape(1, 1, 1, 3)
    with torch.no_grad():
        out = render_rays(enc, field, ren, rs, rd)
    hit = g["svo_hits"][0]
    missed = out["missed"].reshape(-1).cpu().numpy()
    np.testing.assert_allclose(missed[hit], g["render_missed"], atol=2e-4)
    col = out["colors"].reshape(-1, 3).cpu().numpy()
    bg = 1.0
    np.testing.assert_allclose(col[hit], g["render_colors"] + g["render_missed"][:, None] * bg,
                               atol=2e-4)
    assert np.allclose(col[~hit], bg) and np.allclose(missed[~hit], 1.0)


def test_render_gradients_flow_to_embeddings(golden, cuda):
    """Training-mode render: gradients reach the corner embeddings and the
    MLP through the hand-written compositing and scatter kernels, and match a
    float64 autograd render of the same samples."""
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.renderer import VolumeRenderer, render_rays
    g = golden
    enc = _encoder(g, cuda, True)
    field = StandInField(weights=[(torch.from_numpy(g["W%d" % i]), torch.from_numpy(g["b%d" % i]))
                                  for i in range(5)]).to(cuda).eval()
    ren = VolumeRenderer(argparse.Namespace(chunk_size=64)).eval()
    rd = _t(g["ray_dir"], cuda).reshape(1, 1, -1, 3)
    rs = _t(g["ray_start"], cuda).reshape(1, 1, 1, 3)
    out = render_rays(enc, field, ren, rs, rd)
    loss = (out["colors"] ** 2).sum()
    loss.backward()
    gv = enc.values.weight.grad
    assert gv is not None and torch.isfinite(gv).all() and gv.abs().sum() > 0
    assert field.layers[0].weight.grad.abs().sum() > 0
