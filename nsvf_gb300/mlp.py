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

    def reference_bf16(self, emb):
        """torch emulation of the kernel's rounding: bf16 operands, FP32 sums."""
        x = emb.float().to(torch.bfloat16).float()
        for i, (W, b) in enumerate(zip(self.w, self.b)):
            x = x @ W.float().t() + b
            if i < 4:
                x = torch.relu(x).to(torch.bfloat16).float()
        return x
