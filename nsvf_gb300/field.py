"""Field MLP of the workloads and the background field.

StandInField is the workloads' 4 x 128 ReLU MLP on the 32-d voxel embedding,
predicting (sigma, rgb), with the reference field's call convention
(RaidanceField.forward(inputs, outputs) returns `inputs` with 'sigma' and
'texture' added: fairnr/modules/field.py:217-279). Its plain forward is FP32
torch.nn.Linear (cuBLAS, TF32 off); the served renderer runs the same weights
in BF16 on the tensor cores (nsvf_gb300/csrc/mlp_tc.cu).

BackgroundField follows fairnr/modules/implicit.py:15-39 (uniform colour;
with min_color == -1 the colour is mapped from [0, 1] to [-1, 1]).
"""
import torch
import torch.nn as nn


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
