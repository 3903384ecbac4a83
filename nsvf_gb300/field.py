"""Field MLP of the workloads and the background field.

StandInField is the workloads' 4 x 128 ReLU MLP on the 32-d voxel embedding,
predicting (sigma, rgb), with the reference field's call convention
(RaidanceField.forward(inputs, outputs) returns `inputs` with 'sigma' and
'texture' added: fairnr/modules/field.py:217-279). Its plain forward is FP32
torch.nn.Linear (cuBLAS, TF32 off); the served renderer runs the same weights
in BF16 on the tensor cores (nsvf_gb300/csrc/mlp_tc.cu).

BackgroundField follows fairnr/modules/implicit.py:15-39 (uniform colour;
with min_color == -1 the colour is mapped from [0, 1] to [-1, 1]).

RaidanceField and its parts (FCLayer, NeRFPosEmbLinear, ImplicitField,
SignedDistanceField, TextureField) are the reference's field family for
models trained with NSVF, drop-in down to parameter names.
"""
import math
from collections import OrderedDict

import torch
import torch.nn as nn
import torch.nn.functional as F


class BackgroundField(nn.Module):
    def __init__(self, out_dim=3, bg_color="1.0,1.0,1.0", min_color=-1, stop_grad=False,
                 background_depth=5.0):
        super().__init__()
        if out_dim == 3:
            bg = [float(b) for b in bg_color.split(',')] if isinstance(bg_color, str) else [bg_color]
            if min_color == -1:
                bg = [b * 2 - 1 for b in bg]
            if len(bg) == 1:
                bg = bg + bg + bg
            bg = torch.tensor(bg)
        else:
            bg = torch.ones(out_dim).uniform_()
            if min_color == -1:
                bg = bg * 2 - 1
        self.out_dim = out_dim
        self.bg_color = nn.Parameter(bg, requires_grad=not stop_grad)
        self.depth = background_depth

    def forward(self, x, **kwargs):
        return self.bg_color.unsqueeze(0).expand(*x.size()[:-1], self.out_dim)


class StandInField(nn.Module):
    """emb [N, in_dim] -> Linear+ReLU x layers -> Linear(hidden, 4): out[:, 0] is
    sigma, out[:, 1:4] the colour."""

    def __init__(self, in_dim=32, hidden=128, layers=4, weights=None, bg_color="1.0,1.0,1.0",
                 min_color=-1):
        super().__init__()
        dims = [in_dim] + [hidden] * layers + [4]
        self.layers = nn.ModuleList(nn.Linear(a, b) for a, b in zip(dims[:-1], dims[1:]))
        if weights is not None:
            self.load_weights(weights)
        else:
            for lin in self.layers:
                nn.init.xavier_uniform_(lin.weight)
                nn.init.constant_(lin.bias, 0.0)
        self.bg_color = BackgroundField(bg_color=bg_color, min_color=min_color)
        self.in_dim, self.hidden, self.num_layers = in_dim, hidden, layers

    def load_weights(self, weights):
        with torch.no_grad():
            for lin, (W, b) in zip(self.layers, weights):
                lin.weight.copy_(torch.as_tensor(W))
                lin.bias.copy_(torch.as_tensor(b))

    def mlp(self, x):
        for i, lin in enumerate(self.layers):
            x = lin(x)
            if i < len(self.layers) - 1:
                x = torch.relu(x)
        return x

    def forward(self, inputs, outputs=("sigma", "texture")):
        out = self.mlp(inputs["emb"])
        inputs["sigma"] = out[:, 0]
        if "texture" in outputs:
            inputs["texture"] = out[:, 1:4]
        return inputs


# ---------------------------------------------------------------------------
# The reference's field family, for models trained with NSVF (nsvf_base and
# its variants). Constructor arguments, submodule names and parameter names
# are the reference's, so its checkpoints' field state dicts load unchanged;
# the computation is FP32 torch (cuBLAS through nn.Linear, as in the
# reference). The tensor-core kernels cover the 4 x 128 workload field only.

class FCLayer(nn.Module):
    """Linear -> (LayerNorm) -> ReLU as `net` (fairnr/modules/module_utils.py:97-111)."""

    def __init__(self, in_dim, out_dim, with_ln=True):
        super().__init__()
        layers = [nn.Linear(in_dim, out_dim)]
        if with_ln:
            layers.append(nn.LayerNorm([out_dim]))
        layers.append(nn.ReLU())
        self.net = nn.Sequential(*layers)

    def forward(self, x):
        return self.net(x)


class NeRFPosEmbLinear(nn.Module):
    """NeRF positional encoding of in_dim inputs into out_dim = in_dim * 2L
    sin/cos features at frequencies 2^k (times pi unless angular, where the
    input is first mapped through acos), optionally followed by a Linear and
    concatenated with the input (fairnr/modules/module_utils.py:56-95). The
    frequencies are the non-trainable parameter `emb`."""

    def __init__(self, in_dim, out_dim, angular=False, no_linear=False, cat_input=False):
        super().__init__()
        if out_dim % (2 * in_dim) != 0:
            raise ValueError("out_dim must be a multiple of 2 * in_dim")
        L = out_dim // 2 // in_dim
        freq = torch.exp(torch.arange(L, dtype=torch.float) * math.log(2.))
        if not angular:
            freq = freq * math.pi
        self.emb = nn.Parameter(freq, requires_grad=False)
        self.angular = angular
        self.linear = None
        if not no_linear:
            self.linear = nn.Linear(out_dim, out_dim)
            nn.init.xavier_uniform_(self.linear.weight)
            nn.init.constant_(self.linear.bias, 0.0)
        self.in_dim, self.out_dim, self.cat_input = in_dim, out_dim, cat_input

    def forward(self, x):
        if x.size(-1) != self.in_dim:
            raise ValueError("NeRFPosEmbLinear: input width %d != %d" % (x.size(-1), self.in_dim))
        lead = x.size()[:-1]
        y = torch.acos(x.clamp(-1 + 1e-6, 1 - 1e-6)) if self.angular else x
        y = y.unsqueeze(-1) @ self.emb.unsqueeze(0)
        y = torch.cat([torch.sin(y), torch.cos(y)], dim=-1).view(*lead, self.out_dim)
        if self.linear is not None:
            y = self.linear(y)
        return torch.cat([y, x], -1) if self.cat_input else y


def _kaiming_linear(m):
    if type(m) == nn.Linear:
        nn.init.kaiming_normal_(m.weight, a=0.0, nonlinearity='relu', mode='fan_in')


class ImplicitField(nn.Module):
    """num_layers FCLayers (the last an nn.Linear when outmost_linear); the
    input is concatenated back after the layers listed in `skips`
    (fairnr/modules/implicit.py:42-75)."""

    def __init__(self, in_dim, out_dim, hidden_dim, num_layers, outmost_linear=False, with_ln=True,
                 skips=None, spec_init=True):
        super().__init__()
        self.skips = skips
        layers, prev = [], in_dim
        for i in range(num_layers):
            last = i == num_layers - 1
            nxt = out_dim if last else hidden_dim
            layers.append(nn.Linear(prev, nxt) if (last and outmost_linear)
                          else FCLayer(prev, nxt, with_ln=with_ln))
            prev = nxt + (in_dim if (skips is not None and i in skips and not last) else 0)
        self.net = []
        if num_layers > 0:
            self.net = nn.ModuleList(layers)
            if spec_init:
                self.net.apply(_kaiming_linear)

    def forward(self, x):
        y = self.net[0](x)
        for i in range(len(self.net) - 1):
            if self.skips is not None and i in self.skips:
                y = torch.cat((x, y), dim=-1)
            y = self.net[i + 1](y)
        return y


class SignedDistanceField(ImplicitField):
    """Density head: (num_layers - 1) FCLayers, one FCLayer to hidden_dim,
    Linear to 1 (fairnr/modules/implicit.py:100-128; the recurrent variant
    is not supported)."""

    def __init__(self, in_dim, hidden_dim, num_layers=1, recurrent=False, with_ln=True,
                 spec_init=True):
        super().__init__(in_dim, in_dim, in_dim, num_layers - 1, with_ln=with_ln, spec_init=spec_init)
        if recurrent:
            raise NotImplementedError("recurrent SignedDistanceField is not supported")
        self.recurrent = False
        self.hidden_layer = FCLayer(in_dim, hidden_dim, with_ln) if num_layers > 0 else nn.Identity()
        self.output_layer = nn.Linear(hidden_dim if num_layers > 0 else in_dim, 1)

    def forward(self, x, state=None):
        return self.output_layer(self.hidden_layer(x)).squeeze(-1), None


class TextureField(ImplicitField):
    """Colour head: an ImplicitField ending in a Linear to 3 (or 4 with alpha)
    (fairnr/modules/implicit.py:131-139)."""

    def __init__(self, in_dim, hidden_dim, num_layers, with_alpha=False, with_ln=True,
                 spec_init=True):
        super().__init__(in_dim, 4 if with_alpha else 3, hidden_dim, num_layers, outmost_linear=True,
                         with_ln=with_ln, spec_init=spec_init)


class RaidanceField(nn.Module):
    """The reference's radiance field (fairnr/modules/field.py:57-279,
    registered as 'radiance_field'): positional-encoding input filters, a
    feature ImplicitField, a SignedDistanceField density head and a
    TextureField colour head, with the same argument names (inputs_to_density
    such as "emb:6:32", inputs_to_texture such as "feat:0:256, ray:4",
    feature/density/texture_embed_dim, feature_layers, texture_layers,
    nerf_style_mlp, no_layernorm_mlp, feature_field_skip_connect,
    transparent_background, min_color, background_stop_gradient,
    zero_z_steps). forward(inputs, outputs) adds 'feat', 'sigma', 'normal'
    (when asked or used), 'feat_n2' and 'texture' to `inputs`. The
    hypernetwork variant is not supported."""

    def __init__(self, args):
        super().__init__()
        self.args = args
        self.updates = -1
        if getattr(args, "hypernetwork", False):
            raise NotImplementedError("the hypernetwork radiance field is not supported")
        self.chunk_size = getattr(args, "chunk_size", 256) * 256
        self.deterministic_step = getattr(args, "deterministic_step", False)
        self.min_color = getattr(args, "min_color", -1)
        self.trans_bg = getattr(args, "transparent_background", "1.0,1.0,1.0")
        self.sgbg = getattr(args, "background_stop_gradient", False)
        self.bg_color = BackgroundField(bg_color=self.trans_bg, min_color=self.min_color,
                                        stop_grad=self.sgbg)
        self.nerf_style = getattr(args, "nerf_style_mlp", False)
        self.with_ln = not getattr(args, "no_layernorm_mlp", False)
        skip = getattr(args, "feature_field_skip_connect", None)
        self.skips = [skip] if skip is not None else None
        self.den_filters, self.den_ori_dims, self.den_input_dims = self._filters(args.inputs_to_density)
        self.tex_filters, self.tex_ori_dims, self.tex_input_dims = self._filters(args.inputs_to_texture)
        self.den_filters, self.tex_filters = nn.ModuleDict(self.den_filters), nn.ModuleDict(self.tex_filters)
        nerf = self.nerf_style
        feat_dim = self.tex_input_dims[0]
        self.feature_field = ImplicitField(
            sum(self.den_input_dims), feat_dim, args.feature_embed_dim,
            8 if nerf else args.feature_layers + 2, with_ln=False if nerf else self.with_ln,
            skips=[4] if nerf else self.skips, spec_init=not nerf)
        self.predictor = SignedDistanceField(
            feat_dim, args.density_embed_dim, recurrent=False, num_layers=1,
            with_ln=False if nerf else self.with_ln, spec_init=not nerf)
        self.renderer = TextureField(
            sum(self.tex_input_dims), args.texture_embed_dim, 2 if nerf else args.texture_layers + 2,
            with_ln=False if nerf else self.with_ln, spec_init=not nerf)
        if getattr(args, "zero_z_steps", 0) > 0:
            self.register_buffer("zero_z", torch.scalar_tensor(1))
        else:
            self.zero_z = 0

    @staticmethod
    def _filters(spec):
        """"name:pos_dim:base_dim:type, ..." -> (filters, input widths, output
        widths); pos_dim > 0 adds a NeRF positional encoding (type 'a'
        angular, 'b' concatenating the input; 'b' is the default except for
        ray and normal)."""
        filters, ori_dims, out_dims = OrderedDict(), [], []
        for item in spec.split(','):
            p = [a.strip() for a in item.strip().split(':')]
            name = p[0]
            kind = p[3] if len(p) > 3 else ('a' if name in ('ray', 'normal') else 'b')
            pos_dim = int(p[1]) if len(p) > 1 else 0
            base = int(p[2]) if len(p) > 2 else 3
            if pos_dim > 0:
                f = NeRFPosEmbLinear(base, base * pos_dim * 2, angular=(kind == 'a'), no_linear=True,
                                     cat_input=(kind == 'b'))
                out = f.out_dim + (f.in_dim if f.cat_input else 0)
            else:
                f, out = nn.Identity(), base
            filters[name] = f
            ori_dims.append(base)
            out_dims.append(out)
        return filters, ori_dims, out_dims

    def set_num_updates(self, updates):
        self.updates = updates
        if getattr(self.args, "zero_z_steps", 0) <= self.updates:
            self.zero_z = self.zero_z * 0

    @torch.enable_grad()
    def forward(self, inputs, outputs=('sigma', 'texture')):
        if inputs.get('feat', None) is None:
            parts, context = [], None
            for i, name in enumerate(self.den_filters):
                if name not in inputs:
                    raise KeyError("radiance field: input '%s' missing" % name)
                if inputs[name].size(-1) != self.den_ori_dims[i]:
                    raise ValueError("radiance field: %s width %d != %d" % (
                        name, inputs[name].size(-1), self.den_ori_dims[i]))
                f = self.den_filters[name]
                if name == 'context':
                    context = f(inputs[name])
                else:
                    parts.append(f(inputs[name]))
            x = torch.cat(parts, -1)
            if context is not None:
                x = torch.cat([x, context.expand(x.size(0), context.size(1))], -1)
            inputs['feat'] = self.feature_field(x)
        if 'sigma' in outputs:
            inputs['sigma'] = self.predictor(inputs['feat'])[0]
        need_normal = ('normal' not in inputs) and (
            ('texture' in outputs and 'normal' in self.tex_filters) or 'normal' in outputs)
        if need_normal:
            g, = torch.autograd.grad(outputs=inputs['sigma'], inputs=inputs['pos'],
                                     grad_outputs=torch.ones_like(inputs['sigma']),
                                     retain_graph=True, create_graph=True)
            # the reference's sign: the normal is the normalised -gradient
            inputs['normal'] = -g if getattr(self.args, "no_normalize_normal", False) \
                else F.normalize(-g, p=2, dim=1)
        if 'texture' in outputs:
            if self.zero_z == 1:
                inputs['feat'] = inputs['feat'] * 0.0
            inputs['feat_n2'] = (inputs['feat'] ** 2).sum(-1)
            parts = []
            for name in self.tex_filters:
                if name not in inputs:
                    raise KeyError("radiance field: input '%s' missing" % name)
                v = inputs[name].unsqueeze(-1) if name == 'sigma' else inputs[name]
                parts.append(self.tex_filters[name](v))
            inputs['texture'] = self.renderer(torch.cat(parts, -1))
            if self.min_color == 0:
                inputs['texture'] = torch.sigmoid(inputs['texture'])
        return inputs


FIELD_REGISTRY = {"radiance_field": RaidanceField}
