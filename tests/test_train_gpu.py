"""The training step (nsvf_gb300.train: per-chunk recomputation, hand-written
backward through compositing, the field MLP and the trilinear embedding
scatter) on the differentiation workload: the 125,476-voxel c2 shell, 4
views x 2,048 hit pixels, targets from a second embedding set.

* against the reference's own autograd gradient at full size
  (golden_train.npz, tests/golden/make_golden_train.py): same samples, loss,
  every field-parameter gradient and 8,192 corner-embedding gradient rows;
* against float64 finite differences of the oracle render on a 16-ray
  subset whose rays cross at most 50 voxels;
* a batch's backward holds one chunk's activations at a time."""
import argparse

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _c3(cuda, go):
    from nsvf_gb300 import scenes
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    p, vs = scenes.scene_shell(1.0 / 64)
    args = argparse.Namespace(voxel_size=vs, max_hits=64, raymarching_stepsize_ratio=0.125,
                              voxel_embed_dim=32, use_octree=True, deterministic_step=True)
    enc = SparseVoxelEncoder(args, points=p)
    with torch.no_grad():
        enc.values.weight.copy_(scenes.voxel_embeddings(enc.values.weight.shape[0], 32, 0.01, seed=1))
    field = StandInField(weights=scenes.stand_in_mlp_weights(
        seed=2, sigma_scale=float(go["sigma_scale"]), sigma_bias=float(go["sigma_bias"])))
    # the fixture's own rays (recomputing them from the pixel indices is not
    # bit-identical across CPU architectures)
    ro = torch.from_numpy(go["ray_start"]).to(cuda)
    rd = torch.from_numpy(go["ray_dir"]).to(cuda)
    return enc.to(cuda), field.to(cuda), ro, rd


def _close(got, ref, what, rtol=2e-3, atol_frac=2e-4):
    got = got.detach().double().cpu().numpy()
    ref = ref.astype(np.float64)
    np.testing.assert_allclose(got, ref, rtol=rtol, atol=atol_frac * np.abs(ref).max() + 1e-30,
                               err_msg=what)


def test_training_step_matches_reference_autograd(golden_train, cuda):
    from nsvf_gb300 import ext, train
    go = golden_train
    enc, field, ro, rd = _c3(cuda, go)
    target = torch.from_numpy(go["target"]).to(cuda)
    samples = train.sample_rays(enc, ro, rd)
    assert bool(samples[0].all())
    # the same samples (the batch holds no ray that enters two voxels at the
    # same depth, where the reference's unstable sort is free to differ)
    assert int(samples[1].ne(-1).sum()) == int(go["n_samples"])
    torch.cuda.reset_peak_memory_stats(cuda)
    base = torch.cuda.memory_allocated(cuda)
    loss = train.train_step(enc, field, ro, rd, target, samples=samples, chunk_rays=1024)
    peak = torch.cuda.max_memory_allocated(cuda) - base
    ext.check_errors(cuda)
    np.testing.assert_allclose(float(loss), float(go["loss"]), rtol=1e-4)
    for li, lin in enumerate(field.layers):
        _close(lin.weight.grad, go["grad_W%d" % li], "W%d" % li)
        _close(lin.bias.grad, go["grad_b%d" % li], "b%d" % li)
    gv = enc.values.weight.grad
    keys = torch.from_numpy(go["grad_values_keys"]).to(cuda)
    _close(gv[keys], go["grad_values_rows"], "values")
    np.testing.assert_allclose(float(gv.double().norm()), float(go["grad_values_norm"]), rtol=1e-3)
    assert int((gv.abs().sum(-1) > 0).sum()) == int(go["grad_values_touched"])
    # one chunk's activations at a time: far below the whole batch's
    ns = int(go["n_samples"])
    whole_batch = ns * (8 * 32 + 4 * 128 * 2) * 4
    print("training step: %d rays, %d samples, peak %.1f MB (whole-batch activations %.1f MB)"
          % (ro.shape[0], ns, peak / 2 ** 20, whole_batch / 2 ** 20))
    assert peak < whole_batch / 4


def test_training_gradients_match_float64_finite_differences(golden_train, cuda):
    """16 rays of the batch, corner embeddings of the (<= 50) voxels they
    cross: the FP32 analytic gradient vs central differences of the float64
    oracle render of the same samples."""
    from nsvf_gb300 import train
    from oracle import cpu
    go = golden_train
    enc, field, ro, rd = _c3(cuda, go)
    target = torch.from_numpy(go["target"]).to(cuda)
    hits, sidx, depth, dist, xyz = train.sample_rays(enc, ro, rd)
    # 16 rays with few voxels between them
    nvox = torch.tensor([len(torch.unique(r[r != -1])) for r in sidx.cpu()])
    sel = torch.argsort(nvox)[:64:4][:16].sort()[0].to(cuda)
    sub = (hits[sel], sidx[sel], depth[sel], dist[sel], xyz[sel])
    st = enc.precompute(id=None)
    colors = train.render_batch(enc, field, ro[sel], rd[sel], samples=sub, states=st)
    loss = ((colors - target[sel]) ** 2).sum()
    loss.backward()
    gv = enc.values.weight.grad.double().cpu().numpy()
    vid = sidx[sel].cpu().numpy()
    mask = vid != -1
    vox = np.unique(vid[mask])
    assert 0 < len(vox) <= 50
    centers = st["voxel_center_xyz"].detach().cpu().numpy()
    feats = st["voxel_vertex_idx"].cpu().numpy()
    W = [(l.weight.detach().double().cpu().numpy(), l.bias.detach().double().cpu().numpy())
         for l in field.layers]
    d = depth[sel].double().cpu().numpy()
    ds = dist[sel].double().cpu().numpy()
    xyz64 = ro[sel].double().cpu().numpy()[:, None] + rd[sel].double().cpu().numpy()[:, None] * d[..., None]
    tgt = target[sel].double().cpu().numpy()
    vs = float(enc.voxel_size)

    def loss64(values):
        emb = cpu.trilinear_embed(xyz64[mask], vid[mask], centers, feats, values, vs)
        s, c = cpu.mlp_forward(emb, W)
        S = np.zeros(mask.shape)
        C = np.zeros(mask.shape + (3,))
        S[mask], C[mask] = s, c
        o = cpu.composite(S, C, d, ds, mask)
        return ((o["colors"] + o["missed"][:, None] - tgt) ** 2).sum()

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
        assert abs(fd - gv[k, e]) <= 2e-3 * abs(fd) + 1e-5 * np.abs(gv).max(), (k, e, fd, gv[k, e])
