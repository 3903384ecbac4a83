"""Training step of the sparse-voxel renderer (the differentiation workload):
FP32 forward and a hand-written backward with per-chunk recomputation.

The reference trains through autograd and keeps every ray chunk's graph
alive until the loss's backward (fairnr/modules/renderer.py:135-232): the
[samples, 8, 32] corner gathers and every MLP activation of the whole batch.
Here `RayChunk` is one torch.autograd.Function per chunk of rays that keeps
only the chunk's inputs (sample voxel ids, positions, depths, lengths). Its
backward evaluates the chunk again and runs

  compositing backward     nsvf_composite_backward (transmittance prefix
                           recomputed in the kernel)
  free energy backward     d sigma = d fe * dist * 7 where sigma > 0
  MLP backward             per layer, from the saved pre-activations:
                           dW = dZ^T A, db = sum dZ, dA = dZ W, dZ = dA (Z > 0)
                           (FP32 GEMMs, cuBLAS through torch.mm)
  interpolation backward   nsvf_trilinear_embed_backward (float4 atomics
                           into the corner embeddings)

so a batch needs one chunk's activations at a time. The field is the
workloads' 4 x 128 ReLU MLP (field.StandInField); the embeddings are the
encoder's `values` table.

`train_step` renders a batch of rays (intersection, sampling distribution,
inverse-CDF samples: no gradient), takes the squared colour error against
the targets, backpropagates, and applies an optimizer step if one is given.
The sigma noise the reference adds in training mode
(fairnr/modules/renderer.py:119) is left out, as in evaluation mode, so that
gradients are reproducible.
"""
import torch
from torch.autograd import Function

from . import ext
from ._lib import LIB, check
from .functional import composite

SIGMA_SCALE = 7.0     # fairnr/modules/renderer.py:121


def _p(t):
    return t.data_ptr() if t is not None else None


def _interp(vid, xyz, centers, feats, values, voxel_size):
    ns, E = vid.numel(), values.size(-1)
    emb = torch.empty(ns, E, dtype=torch.float32, device=xyz.device)
    if ns:
        check(LIB.nsvf_trilinear_embed(
            ns, E, float(voxel_size), centers.size(0), values.size(0), _p(vid), vid.element_size(),
            _p(xyz), _p(centers), _p(feats), feats.element_size(), _p(values), _p(emb),
            _p(ext.error_word(xyz.device)), ext.ctypes_stream(xyz.device)), "trilinear_embed")
    return emb


def _mlp(emb, params):
    """Forward of the ReLU MLP; returns the output and the per-layer inputs
    A_l and pre-activations Z_l the backward needs."""
    acts, pre = [], []
    x = emb
    n = len(params) // 2
    for l in range(n):
        W, b = params[2 * l], params[2 * l + 1]
        acts.append(x)
        z = torch.addmm(b, x, W.t())
        if l < n - 1:
            pre.append(z)
            x = torch.relu(z)
        else:
            x = z
    return x, acts, pre


class RayChunk(Function):
    """(values, W0, b0, ..., W4, b4, sampled_idx [R, M], xyz [R, M, 3],
    dists [R, M], depths [R, M], centers, feats, voxel_size, kahan)
    -> (colors [R, 3], depth [R], missed [R]) of one chunk of rays."""

    @staticmethod
    def forward(ctx, values, *args):
        params = args[:10]
        sidx, xyz, dists, depths, centers, feats, voxel_size, kahan = args[10:]
        mask = sidx.ne(-1)
        vid = sidx[mask].int().contiguous()
        with torch.no_grad():
            emb = _interp(vid, xyz[mask].contiguous(), centers, feats, values, voxel_size)
            out, _, _ = _mlp(emb, params)
            fe = torch.zeros_like(dists)
            fe[mask] = torch.relu(out[:, 0]) * dists[mask] * SIGMA_SCALE
            tex = torch.zeros(dists.shape + (3,), dtype=torch.float32, device=dists.device)
            tex[mask] = out[:, 1:4]
            _, depth, missed, colors = composite(fe, tex, depths, kahan)
        ctx.save_for_backward(values, *params, sidx, xyz, dists, depths, centers, feats)
        ctx.voxel_size, ctx.kahan = float(voxel_size), bool(kahan)
        return colors, depth, missed

    @staticmethod
    def backward(ctx, g_colors, g_depth, g_missed):
        saved = ctx.saved_tensors
        values, params = saved[0], saved[1:11]
        sidx, xyz, dists, depths, centers, feats = saved[11:]
        dev = dists.device
        mask = sidx.ne(-1)
        vid = sidx[mask].int().contiguous()
        xyz_m = xyz[mask].contiguous()
        with torch.no_grad():
            # the chunk again: interpolation, activations, free energy
            emb = _interp(vid, xyz_m, centers, feats, values, ctx.voxel_size)
            out, acts, pre = _mlp(emb, params)
            sigma = out[:, 0]
            fe = torch.zeros_like(dists)
            fe[mask] = torch.relu(sigma) * dists[mask] * SIGMA_SCALE
            tex = torch.zeros(dists.shape + (3,), dtype=torch.float32, device=dev)
            tex[mask] = out[:, 1:4]
            R, M = fe.shape
            c = lambda g: g.float().contiguous() if g is not None else None
            g_fe = torch.empty_like(fe)
            g_tex = torch.empty_like(tex)
            check(LIB.nsvf_composite_backward(
                R, M, _p(fe), _p(tex), _p(depths.float().contiguous()), None, _p(c(g_depth)),
                _p(c(g_missed)), _p(c(g_colors)), _p(g_fe), _p(g_tex), int(ctx.kahan),
                ext.ctypes_stream(dev)), "composite_backward")
            d_out = torch.empty_like(out)
            d_out[:, 0] = g_fe[mask] * dists[mask] * SIGMA_SCALE * (sigma > 0)
            d_out[:, 1:4] = g_tex[mask]
            grads = [None] * 10
            dz = d_out
            n = len(params) // 2
            for l in range(n - 1, -1, -1):
                W = params[2 * l]
                grads[2 * l] = dz.t().mm(acts[l])
                grads[2 * l + 1] = dz.sum(0)
                da = dz.mm(W)
                if l > 0:
                    dz = da * (pre[l - 1] > 0)
            g_emb = da.contiguous()
            g_values = torch.zeros_like(values)
            if vid.numel():
                check(LIB.nsvf_trilinear_embed_backward(
                    vid.numel(), values.size(-1), ctx.voxel_size, centers.size(0), values.size(0),
                    _p(vid), vid.element_size(), _p(xyz_m), _p(centers), _p(feats),
                    feats.element_size(), _p(values), _p(g_emb), _p(g_values), None,
                    ext.ctypes_stream(dev)), "trilinear_embed_backward")
        return (g_values, *grads) + (None,) * 8


def field_params(field):
    out = []
    for lin in field.layers:
        out += [lin.weight, lin.bias]
    return out


@torch.no_grad()
def sample_rays(encoder, ray_start, ray_dir, states=None):
    """Intersection, the sampling distribution (slot-order sums) and the
    inverse-CDF samples of a batch of rays (ray_start, ray_dir [R, 3]):
    returns (hit mask [R], sampled_idx, depths, dists [R_hit, M], xyz
    [R_hit, M, 3]). No gradient flows through the geometry."""
    if states is None:
        states = encoder.precompute(id=None)
    R = ray_dir.shape[0]
    _, _, inter, hits = encoder.ray_intersect(
        ray_start.reshape(1, 1, -1, 3).expand(1, 1, R, 3).contiguous() if ray_start.dim() == 2
        else ray_start.reshape(1, 1, 1, 3), ray_dir.reshape(1, 1, R, 3),
        {k: (v.unsqueeze(0) if v is not None else None) for k, v in states.items()})
    inter['probs'], inter['steps'] = ext.ray_probs(inter['intersected_voxel_idx'],
                                                   inter['min_depth'], inter['max_depth'],
                                                   encoder.step_size)
    hits = hits.reshape(-1)
    sub = {k: v.reshape(-1, v.shape[-1])[hits] if v.dim() == 3 else v.reshape(-1)[hits]
           for k, v in inter.items()}
    smp = encoder.ray_sample(sub)
    o = ray_start.reshape(-1, 3)
    o = o[hits] if o.shape[0] == R else o.expand(int(hits.sum()), 3)
    d = ray_dir.reshape(-1, 3)[hits]
    xyz = o[:, None, :] + d[:, None, :] * smp['sampled_point_depth'][..., None]
    return hits, smp['sampled_point_voxel_idx'], smp['sampled_point_depth'], \
        smp['sampled_point_distance'], xyz.contiguous()


def render_batch(encoder, field, ray_start, ray_dir, chunk_rays=1024, states=None, kahan=False,
                 samples=None):
    """Colours [R, 3] of a batch of rays through RayChunk (differentiable
    with respect to the encoder's `values` and the field's parameters), with
    the background filled in for missed rays and the missed part of hit
    rays (fairnr/models/nsvf.py:89-110)."""
    if states is None:
        states = encoder.precompute(id=None)
    if samples is None:
        samples = sample_rays(encoder, ray_start, ray_dir, states)
    hits, sidx, depths, dists, xyz = samples
    values = encoder.values.weight
    centers = states['voxel_center_xyz'].float().contiguous()
    feats = states['voxel_vertex_idx'].int().contiguous()
    params = field_params(field)
    R = ray_dir.shape[0]
    bg = field.bg_color.bg_color.float()
    colors_hit, missed_hit = [], []
    n = sidx.shape[0]
    for i in range(0, n, chunk_rays):
        c, _, m = RayChunk.apply(values, *params, sidx[i:i + chunk_rays].contiguous(),
                                 xyz[i:i + chunk_rays].contiguous(),
                                 dists[i:i + chunk_rays].contiguous(),
                                 depths[i:i + chunk_rays].contiguous(), centers, feats,
                                 float(encoder.voxel_size), kahan)
        colors_hit.append(c)
        missed_hit.append(m)
    colors = bg.expand(R, 3).clone()
    if n:
        ch = torch.cat(colors_hit) + torch.cat(missed_hit)[:, None] * bg
        colors = colors.masked_scatter(hits[:, None].expand(R, 3), ch)
    return colors


def train_step(encoder, field, ray_start, ray_dir, target, optimizer=None, chunk_rays=1024,
               states=None, samples=None):
    """One training step: render the batch, loss = sum of squared colour
    errors against `target` [R, 3], backward (per-chunk recomputation,
    hand-written kernels), optimizer step (if given). Returns the loss."""
    if optimizer is not None:
        optimizer.zero_grad(set_to_none=True)
    colors = render_batch(encoder, field, ray_start, ray_dir, chunk_rays, states, samples=samples)
    loss = ((colors - target) ** 2).sum()
    loss.backward()
    if optimizer is not None:
        optimizer.step()
    return loss.detach()
