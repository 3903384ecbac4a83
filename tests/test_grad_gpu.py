"""Differentiation: the drop-in encoder/renderer with the hand-written
backward kernels (compositing, embedding scatter) against the reference's
autograd gradient (golden fixture, same samples and target) and against
float64 finite differences of the oracle render on a 16-ray subset."""
import argparse

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _setup(golden, dev):
    import os, tempfile
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.renderer import VolumeRenderer
    g = golden
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


def _samples(g, dev, sel=None):
    hit = g["svo_hits"][0]
    rd = torch.from_numpy(g["ray_dir"][hit]).to(dev)
    rs = torch.from_numpy(g["ray_start"]).to(dev).reshape(1, 3).expand(rd.shape[0], 3)
    smp = {k: torch.from_numpy(g["svo_det_%s" % k]).to(dev) for k in
           ["sampled_point_depth", "sampled_point_distance", "sampled_point_voxel_idx"]}
    if sel is not None:
        rs, rd = rs[sel], rd[sel]
        smp = {k: v[sel] for k, v in smp.items()}
    return rs.contiguous(), rd.contiguous(), smp


def test_gradients_match_reference_autograd(golden, cuda):
    g = golden
    enc, field, ren = _setup(g, cuda)
    rs, rd, smp = _samples(g, cuda)
    st = enc.precompute(id=None)
    out = ren(enc, field.forward, rs, rd, dict(smp), st)
    tgt = torch.from_numpy(g["grad_target_colors"]).to(cuda)
    loss = ((out["colors"] - tgt) ** 2).sum()
    loss.backward()
    np.testing.assert_allclose(loss.item(), float(g["grad_loss"]), rtol=1e-4)
    gv = enc.values.weight.grad.cpu().numpy()
    ref = g["grad_values"]
    scale = np.abs(ref).max()
    np.testing.assert_allclose(gv, ref, atol=2e-4 * scale, rtol=1e-3)
    for name, lin in [("grad_W0", field.layers[0]), ("grad_W4", field.layers[4])]:
        r = g[name]
        np.testing.assert_allclose(lin.weight.grad.cpu().numpy(), r, atol=2e-4 * np.abs(r).max(),
                                   rtol=1e-3)


def test_gradients_match_float64_finite_differences(golden, cuda):
    """16 rays, the corner embeddings of the (<= 50) voxels they cross: the
    FP32 analytic gradient vs central differences of the float64 oracle."""
    from oracle import cpu
    g = golden
    enc, field, ren = _setup(g, cuda)
    sel = np.arange(0, 16 * 7, 7)[:16]
    rs, rd, smp = _samples(g, cuda, torch.from_numpy(sel))
    st = enc.precompute(id=None)
    out = ren(enc, field.forward, rs, rd, dict(smp), st)
    tgt = torch.from_numpy(g["grad_target_colors"][sel]).to(cuda)
    loss = ((out["colors"] - tgt) ** 2).sum()
    loss.backward()
    gv = enc.values.weight.grad.double().cpu().numpy()

    vid = smp["sampled_point_voxel_idx"].cpu().numpy()
    mask = vid != -1
    vox = np.unique(vid[mask])
    assert len(vox) <= 50
    centers = st["voxel_center_xyz"].detach().cpu().numpy()
    feats = st["voxel_vertex_idx"].cpu().numpy()
    W = [(l.weight.detach().double().cpu().numpy(), l.bias.detach().double().cpu().numpy())
         for l in field.layers]
    d = smp["sampled_point_depth"].double().cpu().numpy()
    dist = smp["sampled_point_distance"].double().cpu().numpy()
    xyz = rs.double().cpu().numpy()[:, None] + rd.double().cpu().numpy()[:, None] * d[..., None]
    target = tgt.double().cpu().numpy()
    vs = float(g["voxel_size"])

    def loss64(values):
        emb = cpu.trilinear_embed(xyz[mask], vid[mask], centers, feats, values, vs)
        s, c = cpu.mlp_forward(emb, W)
        S = np.zeros(mask.shape)
        C = np.zeros(mask.shape + (3,))
        S[mask], C[mask] = s, c
        o = cpu.composite(S, C, d, dist, mask)
        return ((o["colors"] - target) ** 2).sum()

    values = enc.values.weight.detach().double().cpu().numpy()
    keys = np.unique(feats[vox].reshape(-1))
    rng = np.random.RandomState(0)
    cand = [(k, e) for k in keys for e in range(values.shape[1])]
    cand = [cand[i] for i in rng.permutation(len(cand))]
    cand = [c for c in cand if abs(gv[c]) > 1e-3 * np.abs(gv).max()][:40]
    assert len(cand) >= 20
    eps = 1e-6
    for k, e in cand:
        vp, vm = values.copy(), values.copy()
        vp[k, e] += eps
        vm[k, e] -= eps
        fd = (loss64(vp) - loss64(vm)) / (2 * eps)
        assert abs(fd - gv[k, e]) <= 2e-3 * abs(fd) + 1e-5, (k, e, fd, gv[k, e])
