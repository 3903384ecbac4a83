"""Precision study: images of the served (BF16 field) and drop-in (FP32)
paths against a float64 render of the same samples.

The float64 render is the validation oracle on the GPU (FP64 is used nowhere
else). It takes the FP32 geometry both paths share: hit lists, the sampling
distribution, sample depths, distances and voxel ids (bit-identical between
the drop-in and served paths, and to the reference's operation sequence). It
recomputes interpolation, the field MLP and compositing in float64 with
torch:

  emb = sum_k w_k values[feats[v, k]]     (fairnr/modules/encoder.py:584-590)
  fe  = relu(sigma) * dist * 7            (fairnr/modules/renderer.py:117-121)
  p_i = (1 - exp(-fe_i)) exp(-sum_{j<i} fe_j), colour = sum p c + missed * bg.

`report()` gives the max and RMS RGB error and the max depth error (hit
pixels) of each path against it: the served BF16 frame, the served frame with
E4M3 hidden layers, the served chain with the FP32 field, and the drop-in FP32
frame.

Samples far outside their voxel. The reference's inverse-CDF kernel can give
a sample the voxel id of the next row (its tail loop, which this library
reproduces bit for bit: fairnr/clib/src/sample_gpu.cu:188-201). Such a
sample's position lies voxels away from that voxel, and the trilinear weights
extrapolate (by 1e5x at the c2 frame), so field outputs there are orders of
magnitude larger than elsewhere. A relative MLP error then becomes a large
absolute colour error on those pixels; the served chain therefore evaluates
those samples again in double-float arithmetic (nsvf_field_exact_dev). The
report counts these samples (a coordinate more than half a voxel outside the
voxel) and gives the errors over all pixels and over the pixels that have
none.
"""
import torch

from . import ext
from ._lib import LIB, check
from .renderer import render_rays
from .served import SceneState, render_frame


@torch.no_grad()
def fp64_render(encoder, field, ray_start, ray_dir, chunk=32768):
    """Float64 colours [R, 3] and depths [R] of the rays (ray_start [3],
    ray_dir [R, 3] on the encoder's device), on the samples both the drop-in
    and the served paths evaluate (the FP32 geometry: intersection, the
    sampling distribution of nsvf_ray_probs, inverse-CDF placement)."""
    dev = ray_dir.device
    R = ray_dir.shape[0]
    st = encoder.precompute(id=None)
    rs4 = ray_start.reshape(1, 1, 1, 3)
    rd4 = ray_dir.reshape(1, 1, -1, 3)
    _, _, inter, hits = encoder.ray_intersect(rs4, rd4, {k: (v.unsqueeze(0) if v is not None else None)
                                                         for k, v in st.items()})
    hits = hits.reshape(-1)
    pix = hits.nonzero().squeeze(1)
    inter['probs'], inter['steps'] = ext.ray_probs(inter['intersected_voxel_idx'],
                                                   inter['min_depth'], inter['max_depth'],
                                                   encoder.step_size)
    sub = {k: v.reshape(-1, v.shape[-1])[pix] for k, v in inter.items() if k != 'steps'}
    sub['steps'] = inter['steps'].reshape(-1)[pix]
    samples = encoder.ray_sample(sub)
    centers = st['voxel_center_xyz'].double()
    feats = st['voxel_vertex_idx']
    values = st['voxel_vertex_emb'].double()
    W = [(l.weight.double(), l.bias.double()) for l in field.layers]
    bg = field.bg_color.bg_color.double()
    colors = bg.expand(R, 3).clone()
    foreign = torch.zeros(R, dtype=torch.bool, device=dev)
    n_foreign = 0
    depths = torch.full((R,), float(field.bg_color.depth), dtype=torch.float64, device=dev)
    vs = float(encoder.voxel_size)
    cc = torch.tensor([-1.0, 1.0], dtype=torch.float64, device=dev)
    ox, oy, oz = torch.meshgrid([cc, cc, cc], indexing="ij")
    q = (torch.stack([ox.reshape(-1), oy.reshape(-1), oz.reshape(-1)], 1) * .5 + .5)[None]
    o64 = ray_start.double().reshape(1, 1, 3)
    for a in range(0, pix.numel(), chunk):
        b = min(pix.numel(), a + chunk)
        vid = samples['sampled_point_voxel_idx'][a:b].long()
        t = samples['sampled_point_depth'][a:b].double()
        dist = samples['sampled_point_distance'][a:b].double()
        mask = vid.ne(-1)
        rd = ray_dir[pix[a:b]].double()
        xyz = o64 + rd[:, None, :] * t[..., None]
        v = vid[mask]
        p = ((xyz[mask] - centers[v]) / vs + .5)[:, None, :]
        far = ((p[:, 0] < -0.5) | (p[:, 0] > 1.5)).any(-1)
        n_foreign += int(far.sum())
        fr = torch.zeros(mask.shape, dtype=torch.bool, device=dev)
        fr[mask] = far
        foreign[pix[a:b]] = fr.any(-1)
        w = (p * q + (1 - p) * (1 - q)).prod(-1)
        emb = (w[..., None] * values[feats[v]]).sum(1)
        x = emb
        for li, (Wl, bl) in enumerate(W):
            x = x @ Wl.t() + bl
            if li < len(W) - 1:
                x = torch.relu(x)
        sig = torch.zeros(mask.shape, dtype=torch.float64, device=dev)
        rgb = torch.zeros(mask.shape + (3,), dtype=torch.float64, device=dev)
        sig[mask] = x[:, 0]
        rgb[mask] = x[:, 1:4]
        fe = torch.relu(sig) * dist * 7.0 * mask
        sh = torch.cat([fe.new_zeros(fe.shape[0], 1), fe[:, :-1]], 1)
        pr = (1 - torch.exp(-fe)) * torch.exp(-torch.cumsum(sh, 1))
        missed = 1 - pr.sum(-1)
        colors[pix[a:b]] = (rgb * pr[..., None]).sum(1) + missed[:, None] * bg
        depths[pix[a:b]] = (t.masked_fill(~mask, 0) * pr).sum(-1) + missed * float(field.bg_color.depth)
    return colors, depths, hits, foreign, n_foreign


def report(encoder, field, renderer, ray_start, ray_dir):
    """Errors against the float64 render of the served BF16 and FP8 frames,
    the served chain with the FP32 field (all three with the double-float
    pass over samples far outside their voxel), and the drop-in FP32 frame
    (the reference's module structure, no such pass)."""
    ref_c, ref_d, hits, foreign, n_foreign = fp64_render(encoder, field, ray_start, ray_dir)
    scene = SceneState(encoder, field)
    served = render_frame(scene, ray_start, ray_dir)
    served8 = render_frame(scene, ray_start, ray_dir, mlp="tc_fp8")
    chain32 = render_frame(scene, ray_start, ray_dir, mlp="fp32")
    with torch.no_grad():
        plain = render_rays(encoder, field, renderer, ray_start.reshape(1, 1, 1, 3),
                            ray_dir.reshape(1, 1, -1, 3))
    out = {}
    for name, c, d in [
            ("served_bf16", served["colors"], served["depths"]),
            ("served_fp8", served8["colors"], served8["depths"]),
            ("served_fp32", chain32["colors"], chain32["depths"]),
            ("plain_fp32", plain["colors"].reshape(-1, 3), plain["depths"].reshape(-1))]:
        rc, rdp, fr = ref_c, ref_d, foreign
        e = (c.double() - rc).abs()
        de = (d.double() - rdp).abs()[hits]
        clean = e[~fr]
        out[name] = {"max_rgb_err": float(e.max()), "rms_rgb_err": float(e.pow(2).mean().sqrt()),
                     "max_depth_err_hit_pixels": float(de.max()) if de.numel() else 0.0,
                     "max_rgb_err_clean_pixels": float(clean.max()) if clean.numel() else 0.0,
                     "rms_rgb_err_clean_pixels": float(clean.pow(2).mean().sqrt()) if clean.numel() else 0.0}
    out["hit_pixels"] = int(hits.sum())
    out["samples_outside_their_voxel"] = n_foreign
    out["samples_reevaluated_in_double_float"] = int(served["n_far_outside"])
    out["pixels_with_such_samples"] = int(foreign.sum())
    return out
