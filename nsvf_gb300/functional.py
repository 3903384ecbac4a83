"""Differentiable wrappers (torch.autograd.Function) around the
interpolation and compositing kernels, with hand-written backward kernels.

* trilinear_embed(sampled_idx, xyz, centers, feats, values, voxel_size)
    forward  = nsvf_trilinear_embed
    backward = nsvf_trilinear_embed_backward (scatter into the corner
               embeddings with float4 atomics; grad_xyz when xyz needs it)
* composite(free_energy, texture, sampled_depth, kahan=False)
    -> (probs, depth, missed, colors)
    backward = nsvf_composite_backward (recomputes the transmittance prefix
               instead of storing it)
"""
import torch
from torch.autograd import Function

from . import ext
from ._lib import LIB, check


def _p(t):
    return t.data_ptr() if t is not None else None


class TrilinearEmbed(Function):
    @staticmethod
    def forward(ctx, sampled_idx, xyz, centers, feats, values, voxel_size):
        sampled_idx = sampled_idx.contiguous()
        xyz = xyz.float().contiguous()
        centers = centers.float().contiguous()
        feats = feats.contiguous()
        values = values.float().contiguous()
        ns, E = sampled_idx.numel(), values.size(-1)
        emb = torch.empty(ns, E, dtype=torch.float32, device=xyz.device)
        with ext._timed("trilinear_embed", xyz.device):
            check(LIB.nsvf_trilinear_embed(
                ns, E, float(voxel_size), centers.size(0), values.size(0), _p(sampled_idx),
                sampled_idx.element_size(), _p(xyz), _p(centers), _p(feats), feats.element_size(),
                _p(values), _p(emb), _p(ext.error_word(xyz.device)),
                ext.ctypes_stream(xyz.device)), "trilinear_embed")
        ctx.save_for_backward(sampled_idx, xyz, centers, feats, values)
        ctx.voxel_size = float(voxel_size)
        return emb

    @staticmethod
    def backward(ctx, grad_emb):
        sampled_idx, xyz, centers, feats, values = ctx.saved_tensors
        need_xyz, need_values = ctx.needs_input_grad[1], ctx.needs_input_grad[4]
        if not (need_xyz or need_values):
            return None, None, None, None, None, None
        grad_emb = grad_emb.float().contiguous()
        gv = torch.zeros_like(values) if need_values else None
        gx = torch.empty_like(xyz) if need_xyz else None
        check(LIB.nsvf_trilinear_embed_backward(
            sampled_idx.numel(), values.size(-1), ctx.voxel_size, centers.size(0), values.size(0),
            _p(sampled_idx), sampled_idx.element_size(), _p(xyz), _p(centers), _p(feats),
            feats.element_size(), _p(values), _p(grad_emb), _p(gv), _p(gx),
            ext.ctypes_stream(xyz.device)), "trilinear_embed_backward")
        return None, gx, None, None, gv, None


def trilinear_embed(sampled_idx, xyz, centers, feats, values, voxel_size):
    return TrilinearEmbed.apply(sampled_idx, xyz, centers, feats, values, voxel_size)


class Composite(Function):
    @staticmethod
    def forward(ctx, free_energy, texture, sampled_depth, kahan=False):
        fe = free_energy.float().contiguous()
        tex = texture.float().contiguous() if texture is not None else None
        t = sampled_depth.float().contiguous() if sampled_depth is not None else None
        R, M = fe.shape
        dev = fe.device
        probs = torch.empty(R, M, dtype=torch.float32, device=dev)
        depth = torch.empty(R, dtype=torch.float32, device=dev)
        missed = torch.empty(R, dtype=torch.float32, device=dev)
        colors = torch.empty(R, 3, dtype=torch.float32, device=dev)
        with ext._timed("composite", dev):
            check(LIB.nsvf_composite(R, M, _p(fe), _p(tex), _p(t), _p(probs), _p(depth),
                                     _p(missed), _p(colors), int(bool(kahan)),
                                     ext.ctypes_stream(dev)), "composite")
        ctx.save_for_backward(fe, tex, t)
        ctx.kahan = bool(kahan)
        ctx.has_tex = tex is not None
        ctx.mark_non_differentiable()
        return probs, depth, missed, colors

    @staticmethod
    def backward(ctx, g_probs, g_depth, g_missed, g_colors):
        fe, tex, t = ctx.saved_tensors
        R, M = fe.shape
        dev = fe.device
        c = lambda g: g.float().contiguous() if g is not None else None
        g_fe = torch.empty_like(fe)
        g_tex = torch.empty_like(tex) if (tex is not None and ctx.needs_input_grad[1]) else None
        check(LIB.nsvf_composite_backward(
            R, M, _p(fe), _p(tex), _p(t), _p(c(g_probs)), _p(c(g_depth)), _p(c(g_missed)),
            _p(c(g_colors) if tex is not None else None), _p(g_fe), _p(g_tex), int(ctx.kahan),
            ext.ctypes_stream(dev)), "composite_backward")
        return g_fe, g_tex, None, None


def composite(free_energy, texture, sampled_depth, kahan=False):
    return Composite.apply(free_energy, texture, sampled_depth, kahan)
