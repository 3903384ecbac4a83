"""The tcgen05 BF16 field MLP against torch: bit-level agreement with a
torch emulation of its rounding (bf16 operands and activations, FP32 sums)
up to summation order, and the BF16-vs-FP32 error of the field outputs."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


# 128 * 152 * 7 + 5: seven or eight tiles per CTA, so every CTA runs full
# groups of three tile slots (the head-read hand-off between a slot's tiles)
# and a partial last group
@pytest.mark.parametrize("n", [1, 127, 128, 1000, 128 * 300 + 77, 128 * 152 * 7 + 5])
def test_mlp_matches_torch(cuda, n):
    from nsvf_gb300 import ext, scenes
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.mlp import TensorCoreMLP
    torch.manual_seed(n)
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=3)).to(cuda)
    with torch.no_grad():
        for lin in field.layers:
            lin.bias.uniform_(-0.1, 0.1)
    mlp = TensorCoreMLP(field)
    emb = torch.randn(n, 32, device=cuda)
    out = mlp(emb)
    ext.check_errors(cuda)
    emu = mlp.reference_bf16(emb)
    scale = emu.abs().max().item() + 1e-6
    if n < 100000:
        np.testing.assert_allclose(out.cpu().numpy(), emu.cpu().numpy(), atol=2e-3 * scale, rtol=1e-2)
    else:
        # Over 100k samples a few activations round to the neighbouring bf16
        # value (the tensor core sums in another order than torch), which
        # moves that row's outputs by about 1e-3 of the scale; a slot mix-up
        # would spoil whole 128-row tiles instead.
        diff = (out - emu).abs()
        bad = diff > 2e-3 * scale + 1e-2 * emu.abs()
        assert bad.float().mean().item() < 1e-4, int(bad.sum())
        assert diff.max().item() < 2e-2 * scale
    with torch.no_grad():
        f32 = field.mlp(emb)
    err = (out - f32).abs().max().item() / (f32.abs().max().item() + 1e-6)
    assert err < 0.03, err


def test_mlp_repeated_calls_are_deterministic(cuda):
    from nsvf_gb300 import scenes
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.mlp import TensorCoreMLP
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=4)).to(cuda)
    mlp = TensorCoreMLP(field)
    emb = torch.randn(50000, 32, device=cuda)
    a = mlp(emb)
    b = mlp(emb)
    assert torch.equal(a, b)


def test_fused_interpolation_equals_unfused(golden, cuda):
    """Interpolation fused into the MLP input stage gives bit-identical
    outputs to the interpolation kernel followed by the MLP kernel."""
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.functional import trilinear_embed
    from nsvf_gb300.mlp import TensorCoreMLP
    g = golden
    hit = g["svo_hits"][0]
    d = g["svo_det_sampled_point_depth"]
    mask = g["svo_det_sampled_point_voxel_idx"] != -1
    xyz = (g["ray_start"][None, None] + g["ray_dir"][hit][:, None] * d[..., None]).astype(np.float32)[mask]
    n = xyz.shape[0]
    xyzd = torch.zeros(n, 4, device=cuda)
    xyzd[:, :3] = torch.from_numpy(xyz).to(cuda)
    vox = torch.from_numpy(g["svo_det_sampled_point_voxel_idx"][mask]).to(cuda).int()
    centers = torch.from_numpy(g["svo_centers_shifted"]).to(cuda)
    feats = torch.from_numpy(g["feats"]).to(cuda).int()
    values = torch.from_numpy(g["embed"]).to(cuda)
    field = StandInField(weights=[(torch.from_numpy(g["W%d" % i]), torch.from_numpy(g["b%d" % i]))
                                  for i in range(5)]).to(cuda)
    mlp = TensorCoreMLP(field)
    fused = mlp.field_samples(vox, xyzd, centers, feats, values, float(g["voxel_size"]))
    emb = trilinear_embed(vox, xyzd[:, :3], centers, feats, values, float(g["voxel_size"]))
    assert torch.equal(fused, mlp(emb))


@pytest.mark.parametrize("rule,bits", [(0, 16), (1, 8)])
def test_prune_scores_against_reference(golden, golden_prune, cuda, rule, bits):
    """Fused pruning scores vs a torch composition of the same steps (points
    from offset_points, FP32 interpolation kernel, BF16-emulated MLP), and the
    keep mask vs the reference's FP32 mask away from the threshold."""
    from nsvf_gb300 import geometry
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.functional import trilinear_embed
    from nsvf_gb300.mlp import TensorCoreMLP
    g, gp = golden, golden_prune
    vs = float(g["voxel_size"])
    centers = torch.from_numpy(g["svo_centers_shifted"]).to(cuda)
    feats = torch.from_numpy(g["feats"]).to(cuda).int()
    values = torch.from_numpy(g["embed"]).to(cuda)
    field = StandInField(weights=[(torch.from_numpy(g["W%d" % i]), torch.from_numpy(g["b%d" % i]))
                                  for i in range(5)]).to(cuda)
    mlp = TensorCoreMLP(field)
    step = float(gp["step"])
    score = mlp.prune_scores(centers, feats, values, vs, bits=bits, rule=rule, step=step)
    pts = geometry.offset_points(centers, torch.tensor(vs / 2.0, device=cuda), bits=bits)
    idx = torch.arange(centers.size(0), device=cuda)[:, None].expand(*pts.shape[:2]).reshape(-1)
    emb = trilinear_embed(idx, pts.reshape(-1, 3), centers, feats, values, vs)
    sig = mlp.reference_bf16(emb)[:, 0].reshape(centers.size(0), -1)
    if rule == 0:
        ref = torch.exp(-torch.relu(sig)).min(-1)[0]
        ref_keep = gp["keep16"]
        margin = np.abs((1 - gp["minscore16"]) - 0.5)
        keep = ((1 - score) > 0.5).cpu().numpy()
    else:
        ref = (1 - torch.exp(-torch.relu(sig) * step)).max(-1)[0]
        th = float(gp["th8"])
        ref_keep = gp["keep8"]
        margin = np.abs(gp["maxalpha8"] - th)
        keep = (score >= th).cpu().numpy()
    np.testing.assert_allclose(score.cpu().numpy(), ref.cpu().numpy(), rtol=2e-3, atol=2e-4)
    far = margin > 0.02
    assert np.array_equal(keep[far], ref_keep[far])
    assert far.sum() > 0.8 * far.size


def test_fp8_hidden_layers_match_emulation(golden, cuda):
    """E4M3 hidden layers (nsvf_field_samples_fp8) against a torch emulation
    of the same quantisation (per-layer scales, saturating E4M3 rounding,
    FP32 sums). Summation order and one fused multiply-add in the dequantise
    step can flip single E4M3 roundings, so the bar is statistical; the
    error against the FP32 field is reported as the FP8 option's cost."""
    from nsvf_gb300 import scenes
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.functional import trilinear_embed
    from nsvf_gb300.mlp import TensorCoreMLP
    g = golden
    hit = g["svo_hits"][0]
    d = g["svo_det_sampled_point_depth"]
    mask = g["svo_det_sampled_point_voxel_idx"] != -1
    xyz = (g["ray_start"][None, None] + g["ray_dir"][hit][:, None] * d[..., None]).astype(np.float32)[mask]
    n = xyz.shape[0]
    xyzd = torch.zeros(n, 4, device=cuda)
    xyzd[:, :3] = torch.from_numpy(xyz).to(cuda)
    vox = torch.from_numpy(g["svo_det_sampled_point_voxel_idx"][mask]).to(cuda).int()
    centers = torch.from_numpy(g["svo_centers_shifted"]).to(cuda)
    feats = torch.from_numpy(g["feats"]).to(cuda).int()
    values = (torch.from_numpy(g["embed"]) * 50.0).to(cuda)      # activations well inside E4M3
    vs = float(g["voxel_size"])
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=5)).to(cuda)
    with torch.no_grad():
        for lin in field.layers:
            lin.bias.uniform_(-0.05, 0.05)
    mlp = TensorCoreMLP(field)
    emb = trilinear_embed(vox, xyzd[:, :3], centers, feats, values, vs)
    mlp.enable_fp8(emb)
    out = mlp.field_samples_fp8(vox, xyzd, centers, feats, values, vs)
    from nsvf_gb300 import ext
    ext.check_errors(cuda)
    emu = mlp.reference_fp8(emb)
    with torch.no_grad():
        f32 = field.mlp(emb)
    scale = f32.abs().max().item()
    diff = (out - emu).abs() / scale
    err32 = (out - f32).abs() / scale
    stats = dict(n=n, median_vs_emulation=diff.median().item(), max_vs_emulation=diff.max().item(),
                 max_vs_fp32=err32.max().item(), rms_vs_fp32=err32.pow(2).mean().sqrt().item())
    print("fp8 hidden layers:", stats)
    assert n > 5000
    assert stats["median_vs_emulation"] <= 2e-3, stats
    assert stats["max_vs_emulation"] <= 5e-2, stats
    assert stats["max_vs_fp32"] <= 0.15, stats


def test_bounded_wait_times_out_and_leaves_the_context_usable(cuda):
    """The tensor-core kernels' waits are bounded: a wait on an mbarrier
    phase that never completes gives up after its limit, records bit 3 (8)
    in the error word and returns; the next launch runs normally."""
    import time
    from nsvf_gb300 import ext, scenes
    from nsvf_gb300._lib import LIB
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.mlp import TensorCoreMLP
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    t0 = time.perf_counter()
    assert LIB.nsvf_wait_timeout_selftest(2_000_000, err.data_ptr(), ext.ctypes_stream(cuda)) == 0
    torch.cuda.synchronize(cuda)
    assert time.perf_counter() - t0 < 5.0
    assert int(err.item()) == 8
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=3)).to(cuda)
    mlp = TensorCoreMLP(field)
    emb = torch.randn(1000, 32, device=cuda)
    out = mlp(emb)
    ext.check_errors(cuda)
    np.testing.assert_allclose(out.cpu().numpy(), mlp.reference_bf16(emb).cpu().numpy(),
                               atol=2e-3 * (out.abs().max().item() + 1e-6), rtol=1e-2)
