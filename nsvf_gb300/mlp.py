"""Tensor-core field MLP (nsvf_mlp_forward_bf16) for the StandInField weights.

TensorCoreMLP(field) snapshots the field's weights as bf16 (row-major
[out, in]) and biases as FP32 on the field's device; calling it on an FP32
embedding [N, 32] returns [N, 4] = (sigma, r, g, b) in FP32.
"""
import ctypes

import torch

from . import ext
from ._lib import LIB, check


class TensorCoreMLP:
    def __init__(self, field):
        dims = [(lin.out_features, lin.in_features) for lin in field.layers]
        if dims != [(128, 32), (128, 128), (128, 128), (128, 128), (4, 128)]:
            raise ValueError("tensor-core MLP supports the 32-128x4-4 field, got %s" % dims)
        self.w = [lin.weight.detach().to(torch.bfloat16).contiguous() for lin in field.layers]
        self.b = [lin.bias.detach().float().contiguous() for lin in field.layers]
        self.device = self.w[0].device
        self._wp = (ctypes.c_void_p * 5)(*[t.data_ptr() for t in self.w])
        self._bp = (ctypes.c_void_p * 5)(*[t.data_ptr() for t in self.b])

    def __call__(self, emb, out=None):
        emb = emb.float().contiguous()
        n = emb.shape[0]
        if out is None:
            out = torch.empty(n, 4, dtype=torch.float32, device=emb.device)
        with ext._timed("mlp_forward_bf16", emb.device):
            check(LIB.nsvf_mlp_forward_bf16(n, emb.data_ptr(), self._wp, self._bp, out.data_ptr(),
                                            ext.error_word(emb.device).data_ptr(),
                                            ext.ctypes_stream(emb.device)), "mlp_forward_bf16")
        return out

    def field_samples(self, voxel, xyz_dist, centers, feats, values, voxel_size, out=None):
        """Fused interpolation + MLP on compacted samples: voxel [n] int32,
        xyz_dist [n, 4], centers [V, 3], feats [V, 8] int32, values [Kc, 32]
        -> [n, 4] (sigma, r, g, b)."""
        n = voxel.numel()
        dev = voxel.device
        if out is None:
            out = torch.empty(n, 4, dtype=torch.float32, device=dev)
        with ext._timed("field_samples_bf16", dev):
            check(LIB.nsvf_field_samples_bf16(
                n, voxel.data_ptr(), xyz_dist.data_ptr(), centers.size(0), values.size(0),
                float(voxel_size), centers.data_ptr(), feats.data_ptr(), values.data_ptr(),
                self._wp, self._bp, out.data_ptr(), ext.error_word(dev).data_ptr(),
                ext.ctypes_stream(dev)), "field_samples_bf16")
        return out

    def prune_scores(self, centers, feats, values, voxel_size, bits=8, rule=1, step=0.0):
        """Per-voxel pruning score over bits^3 points (see nsvf_prune_scores_bf16):
        rule 0 -> min exp(-relu sigma), rule 1 -> max 1 - exp(-relu(sigma) step)."""
        V = centers.size(0)
        dev = centers.device
        init = 0x7F800000 if rule == 0 else 0
        score = torch.full((V,), init, dtype=torch.int32, device=dev)
        with ext._timed("prune_scores_bf16", dev):
            check(LIB.nsvf_prune_scores_bf16(
                V, int(bits), int(rule), float(step), values.size(0), float(voxel_size),
                centers.data_ptr(), feats.data_ptr(), values.data_ptr(), self._wp, self._bp,
                score.data_ptr(), ext.error_word(dev).data_ptr(), ext.ctypes_stream(dev)),
                "prune_scores_bf16")
        return score.view(torch.float32)

    def reference_bf16(self, emb):
        """torch emulation of the kernel's rounding: bf16 operands, FP32 sums."""
        x = emb.float().to(torch.bfloat16).float()
        for i, (W, b) in enumerate(zip(self.w, self.b)):
            x = x @ W.float().t() + b
            if i < 4:
                x = torch.relu(x).to(torch.bfloat16).float()
        return x
