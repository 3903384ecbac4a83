"""Precision study: images of the served (BF16 field) and drop-in (FP32)
paths against a float64 render of the same samples.

The float64 render is the validation oracle on the GPU (FP64 is used nowhere
else). It takes the FP32 geometry of the path it checks: hit lists, sample
depths, distances and voxel ids. For the drop-in path that geometry is
bit-identical to the reference's operation sequence; the served path's
differs only in the order of the per-ray sum that sets its sampling
distribution, so it gets a float64 render of its own samples. The render
recomputes interpolation, the field MLP and compositing in float64 with
torch:

  emb = sum_k w_k values[feats[v, k]]     (fairnr/modules/encoder.py:584-590)
  fe  = relu(sigma) * dist * 7            (fairnr/modules/renderer.py:117-121)
  p_i = (1 - exp(-fe_i)) exp(-sum_{j<i} fe_j), colour = sum p c + missed * bg.

`report()` gives the max and RMS RGB error and the max depth error (hit
pixels) of each path against it: the served BF16 frame, the served frame with
E4M3 hidden layers, and the drop-in FP32 frame.

Samples far outside their voxel. The reference's inverse-CDF kernel can give
a sample the voxel id of the next row (its tail loop, which this library
reproduces bit for bit: fairnr/clib/src/sample_gpu.cu:188-201). Such a
sample's position lies voxels away from that voxel, and the trilinear weights
extrapolate (by 1e5x at the c2 frame), so field outputs there are orders of
magnitude larger than elsewhere. A relative MLP error then becomes a large
absolute colour error on those pixels. The report counts these samples (a
coordinate more than half a voxel outside the voxel) and gives the errors
over all pixels and over the pixels that have none.
"""
import torch

from . import ext
from ._lib import LIB, check
from .renderer import render_rays
from .served import SceneState, render_frame


def _served_rows(inter, pix, step_size):
    """The hit rows of rays `pix` with the served path's sampling
    distribution (nsvf_gather_probs: the per-ray sum in its fixed warp
    order)."""
    idx = inter['intersected_voxel_idx']
    H = idx.size(-1)
    dev = idx.device
    idx = idx.reshape(-1, H).int().contiguous()
    lo = inter['min_depth'].reshape(-1, H).float().contiguous()
    hi = inter['max_depth'].reshape(-1, H).float().contiguous()
    n = pix.numel()
    n_dev = torch.tensor([n], dtype=torch.int64, device=dev)
    I = torch.empty(n, H, dtype=torch.int32, device=dev)
    L, U, probs = (torch.empty(n, H, device=dev) for _ in range(3))
    steps = torch.empty(n, device=dev)
    check(LIB.nsvf_gather_probs(n, n_dev.data_ptr(), H, float(step_size), pix.data_ptr(),
                                idx.data_ptr(), lo.data_ptr(), hi.data_ptr(), I.data_ptr(),
                                L.data_ptr(), U.data_ptr(), probs.data_ptr(), steps.data_ptr(),
                                ext.ctypes_stream(dev)), "gather_probs")
    return {'intersected_voxel_idx': I, 'min_depth': L, 'max_depth': U, 'probs': probs,
            'steps': steps}


@torch.no_grad()
def fp64_render(encoder, field, ray_start, ray_dir, chunk=32768, served=False):
    """Float64 colours [R, 3] and depths [R] of the rays (ray_start [3],
    ray_dir [R, 3] on the encoder's device). served: sample with the served
    path's distribution (its per-ray sum order) instead of the drop-in
    path's, so that the samples are the served frame's own."""
    dev = ray_dir.device
    R = ray_dir.shape[0]
    st = encoder.precompute(id=None)
    rs4 = ray_start.reshape(1, 1, 1, 3)
    rd4 = ray_dir.reshape(1, 1, -1, 3)
    _, _, inter, hits = encoder.ray_intersect(rs4, rd4, {k: (v.unsqueeze(0) if v is not None else None)
                                                         for k, v in st.items()})
    hits = hits.reshape(-1)
    pix = hits.nonzero().squeeze(1)
    if served:
        sub = _served_rows(inter, pix, encoder.step_size)
    else:
        d = (inter['max_depth'] - inter['min_depth']).masked_fill(inter['intersected_voxel_idx'].eq(-1), 0)
        inter['probs'] = d / d.sum(-1, keepdim=True)
        inter['steps'] = d.sum(-1) / encoder.step_size
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
    """Errors of the served BF16 and FP8 frames and of the drop-in FP32 frame,
    each against a float64 render of its own samples."""
    ref_c, ref_d, hits, foreign, n_foreign = fp64_render(encoder, field, ray_start, ray_dir)
    srv_c, srv_d, _, srv_foreign, _ = fp64_render(encoder, field, ray_start, ray_dir, served=True)
    scene = SceneState(encoder, field)
    served = render_frame(scene, ray_start, ray_dir)
    served8 = render_frame(scene, ray_start, ray_dir, mlp="tc_fp8")
    with torch.no_grad():
        plain = render_rays(encoder, field, renderer, ray_start.reshape(1, 1, 1, 3),
                            ray_dir.reshape(1, 1, -1, 3))
    out = {}
    for name, c, d, rc, rdp, fr in [
            ("served_bf16", served["colors"], served["depths"], srv_c, srv_d, srv_foreign),
            ("served_fp8", served8["colors"], served8["depths"], srv_c, srv_d, srv_foreign),
            ("plain_fp32", plain["colors"].reshape(-1, 3), plain["depths"].reshape(-1), ref_c, ref_d,
             foreign)]:
        e = (c.double() - rc).abs()
        de = (d.double() - rdp).abs()[hits]
        clean = e[~fr]
        out[name] = {"max_rgb_err": float(e.max()), "rms_rgb_err": float(e.pow(2).mean().sqrt()),
                     "max_depth_err_hit_pixels": float(de.max()) if de.numel() else 0.0,
                     "max_rgb_err_clean_pixels": float(clean.max()) if clean.numel() else 0.0,
                     "rms_rgb_err_clean_pixels": float(clean.pow(2).mean().sqrt()) if clean.numel() else 0.0}
    out["hit_pixels"] = int(hits.sum())
    out["samples_outside_their_voxel"] = n_foreign
    out["pixels_with_such_samples"] = int(foreign.sum())
    return out
