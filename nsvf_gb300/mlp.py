"""Tensor-core field MLP (nsvf_mlp_forward_bf16) for the StandInField weights.

TensorCoreMLP(field) snapshots the field's weights as bf16 (row-major
[out, in]) and biases as FP32 on the field's device; calling it on an FP32
embedding [N, 32] returns [N, 4] = (sigma, r, g, b) in FP32.

enable_fp8(calibration_emb) adds the FP8 option of the fused sample kernel
(nsvf_field_samples_fp8): the three 128x128 hidden layers in E4M3 with
per-layer scales, the input layer and the (sigma, rgb) head in BF16.
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
        self.w32 = [lin.weight.detach().float().contiguous() for lin in field.layers]
        self.fp8 = None

    E4M3_MAX = 448.0

    def enable_fp8(self, calibration_emb):
        """Per-layer scales for E4M3 hidden layers. Weights: w_scale[l] =
        448 / max|W_l|. Activations: a_scale[l] = 448 / (max of the FP32
        activation entering layer l on `calibration_emb` [N, 32]); larger
        values saturate to 448 at run time."""
        x = calibration_emb.float()
        amax = []
        with torch.no_grad():
            for i in range(3):
                x = torch.relu(x @ self.w32[i].t() + self.b[i])
                amax.append(float(x.abs().max()))
        w_scale = [self.E4M3_MAX / max(float(self.w32[l].abs().max()), 1e-30) for l in (1, 2, 3)]
        a_scale = [self.E4M3_MAX / max(a, 1e-30) for a in amax]
        w8 = [(self.w32[l] * s).clamp(-self.E4M3_MAX, self.E4M3_MAX).to(torch.float8_e4m3fn)
              .contiguous() for l, s in zip((1, 2, 3), w_scale)]
        ptrs = [self.w[0].data_ptr()] + [t.data_ptr() for t in w8] + [self.w[4].data_ptr()]
        self.fp8 = {"w8": w8, "w_scale": w_scale, "a_scale": a_scale,
                    "wp": (ctypes.c_void_p * 5)(*ptrs),
                    "scales": (ctypes.c_float * 6)(*(w_scale + a_scale))}
        return self

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

    def field_samples_fp8(self, voxel, xyz_dist, centers, feats, values, voxel_size, out=None):
        """field_samples with E4M3 hidden layers (enable_fp8 first)."""
        if self.fp8 is None:
            raise RuntimeError("TensorCoreMLP.enable_fp8 has not been called")
        n = voxel.numel()
        dev = voxel.device
        if out is None:
            out = torch.empty(n, 4, dtype=torch.float32, device=dev)
        with ext._timed("field_samples_fp8", dev):
            check(LIB.nsvf_field_samples_fp8(
                n, voxel.data_ptr(), xyz_dist.data_ptr(), centers.size(0), values.size(0),
                float(voxel_size), centers.data_ptr(), feats.data_ptr(), values.data_ptr(),
                self.fp8["wp"], self._bp, self.fp8["scales"], out.data_ptr(),
                ext.error_word(dev).data_ptr(), ext.ctypes_stream(dev)), "field_samples_fp8")
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

    def reference_fp8(self, emb):
        """torch emulation of the FP8 kernel: bf16 input layer; the
        accumulator of layer l starts at bias / dq (dq = 1 / (a_scale *
        w_scale) of the layer, 1 for layer 0; float32 scalars as the library
        computes them); for layers 0-2 the output relu(acc * dq * qs) (qs =
        a_scale of the next layer) rounded to saturating E4M3, E4M3 weights;
        layer 3 relu(acc * dq) in bf16; bf16 head."""
        import numpy as np
        f = self.fp8
        f32 = np.float32
        e4 = torch.float8_e4m3fn
        ws = [f32(x) for x in f["w_scale"]]
        as_ = [f32(x) for x in f["a_scale"]]
        dq = [f32(1.0)] + [f32(f32(1.0) / f32(ws[l - 1] * as_[l - 1])) for l in (1, 2, 3)]
        qs = as_ + [f32(1.0)]
        x = emb.float().to(torch.bfloat16).float() @ self.w[0].float().t()
        for l in range(4):
            z = x + self.b[l].float() / float(dq[l])
            if l < 3:
                y = z * float(f32(dq[l] * qs[l]))
                x = torch.relu(y).clamp(max=self.E4M3_MAX).to(e4).float()
                x = x @ f["w8"][l].float().t()
            else:
                x = torch.relu(z * float(dq[3])).to(torch.bfloat16).float()
        return x @ self.w[4].float().t() + self.b[4]
