"""The reference's field family (RaidanceField and its parts) against the
reference's own modules, on the CPU: the reference field's state dict loads
into ours with strict name and shape checks, and the forward pass gives the
same feature, density, normal and texture (same FP32 torch operations, so
bit for bit). Runs where the reference checkout is present."""
import argparse

import pytest
import torch

from oracle import ref_import

pytestmark = pytest.mark.skipif(not ref_import.available(), reason="reference checkout not present")


def _args(**kw):
    a = dict(inputs_to_density="emb:6:32", inputs_to_texture="feat:0:256, ray:4",
             feature_embed_dim=256, density_embed_dim=128, texture_embed_dim=256, feature_layers=1,
             texture_layers=3, background_stop_gradient=False)
    a.update(kw)
    return argparse.Namespace(**a)


@pytest.mark.parametrize("variant", ["nsvf_base", "nerf_style", "no_layernorm", "normal_sigmoid",
                                     "skip_connect"])
def test_radiance_field_matches_reference(variant):
    from nsvf_gb300.field import RaidanceField
    ref = ref_import.load()
    kw = {
        "nsvf_base": {},
        "nerf_style": {"nerf_style_mlp": True},
        "no_layernorm": {"no_layernorm_mlp": True},
        "normal_sigmoid": {"inputs_to_texture": "feat:0:256, normal:4, ray:4", "min_color": 0,
                           "inputs_to_density": "emb:6:32, pos:4"},
        "skip_connect": {"feature_layers": 4, "feature_field_skip_connect": 2},
    }[variant]
    torch.manual_seed(0)
    theirs = ref.field.RaidanceField(_args(**kw))
    ours = RaidanceField(_args(**kw))
    missing = ours.load_state_dict(theirs.state_dict(), strict=True)
    assert not missing.missing_keys and not missing.unexpected_keys
    N = 500
    g = torch.Generator().manual_seed(1)
    emb = torch.randn(N, 32, generator=g)
    ray = torch.nn.functional.normalize(torch.randn(N, 3, generator=g), dim=-1)
    pos = (torch.rand(N, 3, generator=g) * 2 - 1).requires_grad_(True)
    outs = ['sigma', 'texture'] + (['normal'] if variant == "normal_sigmoid" else [])
    a = theirs({"emb": emb.clone(), "ray": ray.clone(), "pos": pos}, outputs=outs)
    b = ours({"emb": emb.clone(), "ray": ray.clone(), "pos": pos}, outputs=outs)
    for k in ["feat", "sigma", "texture", "feat_n2"] + (["normal"] if variant == "normal_sigmoid" else []):
        assert torch.equal(a[k], b[k]), k
    # the background field is the same module as well
    assert torch.equal(theirs.bg_color.bg_color, ours.bg_color.bg_color)
