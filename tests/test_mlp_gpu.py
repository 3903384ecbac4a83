"""The tcgen05 BF16 field MLP against torch: bit-level agreement with a
torch emulation of its rounding (bf16 operands and activations, FP32 sums)
up to summation order, and the BF16-vs-FP32 error of the field outputs."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 127, 128, 1000, 128 * 300 + 77])
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
    np.testing.assert_allclose(out.cpu().numpy(), emu.cpu().numpy(), atol=2e-3 * scale, rtol=1e-2)
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
