"""Drop-in VolumeRenderer (fairnr/modules/renderer.py:51-252) and the
NSVF model glue around the encoder (fairnr/models/nsvf.py:43-110,
fairnr/models/fairnr_model.py:142-186) for one frame of rays.

VolumeRenderer keeps the reference's interface and results; the field is
evaluated once on all valid samples of a ray chunk (the reference walks the
sample columns with a host synchronisation per column), and the compositing
runs in one kernel per chunk (nsvf_composite, hand-written backward). With
raymarching_tolerance > 0 the reference's column-chunk early stop is
reproduced step for step, since it decides which samples are evaluated.
"""
import math
from collections import defaultdict

import torch

from .ext import ray_probs
from .functional import composite
from .geometry import fill_in, ray

MAX_DEPTH = 10000.0


class VolumeRenderer(torch.nn.Module):

    def __init__(self, args):
        super().__init__()
        self.args = args
        self.chunk_size = 1024 * getattr(args, "chunk_size", 64)
        self.valid_chunk_size = 1024 * getattr(args, "valid_chunk_size", self.chunk_size // 1024)
        self.discrete_reg = getattr(args, "discrete_regularization", False)
        self.raymarching_tolerance = getattr(args, "raymarching_tolerance", 0.0)
        self.trace_normal = getattr(args, "trace_normal", False)
        self.sigma_scale = 7.0        # fairnr/modules/renderer.py:121
        self.kahan = getattr(args, "kahan_transmittance", False)

    @staticmethod
    def add_args(parser):
        parser.add_argument('--discrete-regularization', action='store_true')
        parser.add_argument('--chunk-size', type=int, metavar='D')
        parser.add_argument('--valid-chunk-size', type=int, metavar='D')
        parser.add_argument('--raymarching-tolerance', type=float, default=0)
        parser.add_argument('--trace-normal', action='store_true')
        parser.add_argument('--kahan-transmittance', action='store_true')

    def _field(self, input_fn, field_fn, ray_start, ray_dir, samples, encoder_states, mask,
               output_types):
        """Evaluate the field on the masked samples; returns free energy and
        texture scattered back to [R, M] (zeros where masked)."""
        sampled_depth = samples['sampled_point_depth']
        R, M = sampled_depth.shape
        fe = sampled_depth.new_zeros(R, M)
        tex = sampled_depth.new_zeros(R, M, 3) if 'texture' in output_types else None
        n = int(mask.sum())
        if n == 0:
            return fe, tex, 0
        xyz = ray(ray_start.unsqueeze(1), ray_dir.unsqueeze(1), sampled_depth.unsqueeze(2))
        d = ray_dir.unsqueeze(1).expand(R, M, 3)
        sub = {'sampled_point_xyz': xyz[mask], 'sampled_point_ray_direction': d[mask]}
        for k, v in samples.items():
            sub[k] = v[mask]
        inputs = input_fn(sub, encoder_states)
        out = field_fn(inputs, outputs=output_types)
        sigma, dists = out['sigma'], inputs['dists']
        noise = 0 if not self.discrete_reg and (not self.training) else torch.zeros_like(sigma).normal_()
        free_energy = torch.relu(noise + sigma) * dists * self.sigma_scale
        fe = fe.masked_scatter(mask, free_energy)
        if tex is not None:
            tex = tex.masked_scatter(mask.unsqueeze(-1).expand(R, M, 3), out['texture'])
        return fe, tex, n

    def forward_chunk(self, input_fn, field_fn, ray_start, ray_dir, samples, encoder_states,
                      gt_depths=None, output_types=['sigma', 'texture'], global_weights=None):
        sampled_depth = samples['sampled_point_depth']
        sampled_idx = samples['sampled_point_voxel_idx'].long()
        hits = sampled_idx.ne(-1)
        tol = self.raymarching_tolerance
        if tol > 0:
            fe, tex, evals, hits = self._early_stop(input_fn, field_fn, ray_start, ray_dir, samples,
                                                    encoder_states, output_types, -math.log(tol))
        else:
            fe, tex, evals = self._field(input_fn, field_fn, ray_start, ray_dir, samples,
                                         encoder_states, hits, output_types)
        probs, depth_unused, missed, colors = composite(fe, tex, sampled_depth, self.kahan)
        if global_weights is not None:
            probs = probs * global_weights
            missed = 1 - probs.sum(-1)
        depth = (sampled_depth * probs).sum(-1)
        results = {
            'probs': probs, 'depths': depth,
            'max_depths': sampled_depth.masked_fill(hits.eq(0), -1).max(1).values,
            'min_depths': sampled_depth.min(1).values,
            'missed': missed, 'ae': evals,
        }
        if tex is not None:
            results['colors'] = colors if global_weights is None else \
                (tex * probs.unsqueeze(-1)).sum(-2)
        return results

    def _early_stop(self, input_fn, field_fn, ray_start, ray_dir, samples, encoder_states,
                    output_types, tolerance):
        """The reference's column-chunk loop with early termination
        (fairnr/modules/renderer.py:146-188): identical chunk boundaries, so
        the same samples are evaluated."""
        sampled_depth = samples['sampled_point_depth']
        sampled_idx = samples['sampled_point_voxel_idx'].long()
        R, M = sampled_depth.shape
        chunk_size = self.chunk_size if self.training else self.valid_chunk_size
        hits = sampled_idx.ne(-1).long()
        fe_all = sampled_depth.new_zeros(R, M)
        tex_all = sampled_depth.new_zeros(R, M, 3) if 'texture' in output_types else None
        early_stop = None
        acc_fe = 0
        evals = 0
        size_so_far, start = 0, 0
        for i in range(M + 1):
            if ((i == M) or (size_so_far + hits[:, i].sum() > chunk_size)) and (i > start):
                sub = {k: v[:, start:i] for k, v in samples.items()}
                mask = sub['sampled_point_voxel_idx'].ne(-1)
                if early_stop is not None:
                    mask = mask & (~early_stop.unsqueeze(-1))
                fe, tex, n = self._field(input_fn, field_fn, ray_start, ray_dir, sub, encoder_states,
                                         mask, output_types)
                if n > 0:
                    evals += n
                    fe_all[:, start:i] = fe
                    if tex_all is not None:
                        tex_all[:, start:i] = tex
                    acc_fe = acc_fe + fe.sum(1)
                    early_stop = acc_fe > tolerance
                    hits[early_stop] *= 0
                start, size_so_far = i, 0
            if i < M:
                size_so_far += hits[:, i].sum()
        return fe_all, tex_all, evals, hits.bool()

    def forward(self, input_fn, field_fn, ray_start, ray_dir, samples, *args, **kwargs):
        chunk_size = self.chunk_size if self.training else self.valid_chunk_size
        if ray_start.size(0) <= chunk_size:
            results = self.forward_chunk(input_fn, field_fn, ray_start, ray_dir, samples, *args, **kwargs)
        else:
            results = [
                self.forward_chunk(input_fn, field_fn, ray_start[i:i + chunk_size],
                                   ray_dir[i:i + chunk_size],
                                   {name: s[i:i + chunk_size] for name, s in samples.items()},
                                   *args, **kwargs)
                for i in range(0, ray_start.size(0), chunk_size)]
            # chunks may differ in width: pad per-sample outputs before concatenating
            out = {}
            for name in results[0]:
                vals = [r[name] for r in results]
                if isinstance(vals[0], torch.Tensor) and vals[0].dim() > 1:
                    W = max(v.size(1) for v in vals)
                    vals = [torch.nn.functional.pad(v, (0, W - v.size(1))) for v in vals]
                    out[name] = torch.cat(vals, 0)
                elif isinstance(vals[0], torch.Tensor) and vals[0].dim() > 0:
                    out[name] = torch.cat(vals, 0)
                else:
                    out[name] = sum(vals)
            results = out
        if getattr(input_fn, "track_max_probs", False) and (not self.training):
            input_fn.track_voxel_probs(samples['sampled_point_voxel_idx'].long(), results['probs'])
        return results


def normalize_rows(x):
    """x / x.sum(-1) with each row summed one slot at a time in slot order
    (nsvf_ray_probs on intervals [0, x]), the order the sampling
    distributions of this library use."""
    H = x.size(-1)
    idx = torch.zeros(x.shape, dtype=torch.int32, device=x.device)
    p, tot = ray_probs(idx, torch.zeros_like(x, dtype=torch.float32), x.float(), 1.0)
    return p, tot


def prepare_hierarchical_sampling(intersection_outputs, samples, all_results,
                                  fixed_fine_num_samples=0, reduce_fine_for_missed=False,
                                  fine_num_sample_ratio=0):
    """Hierarchical resampling (fairnr/models/nerf.py:64-79; NSVFModel's
    fine_num_sample_ratio, fairnr/models/nsvf.py:83-87): every coarse sample
    becomes an interval [t - d/2, t + d/2] with its voxel id; the
    distribution is the coarse render's per-sample probs plus 1e-5,
    normalised per ray (slot-order sum); steps are 1 per ray times
    fixed_fine_num_samples (if set), times the ray's summed probs with
    reduce_fine_for_missed, or fine_num_sample_ratio times the ray's number
    of coarse samples (if set, NSVF's rule). The inverse-CDF op then places
    the fine samples."""
    depth = samples.get('original_point_depth', samples['sampled_point_depth'])
    dists = samples.get('original_point_distance', samples['sampled_point_distance'])
    out = dict(intersection_outputs)
    out['min_depth'] = depth - dists * .5
    out['max_depth'] = depth + dists * .5
    out['intersected_voxel_idx'] = samples['sampled_point_voxel_idx'].contiguous()
    safe = all_results['probs'] + 1e-5
    out['probs'], total = normalize_rows(safe)
    out['steps'] = safe.new_ones(*safe.size()[:-1])
    if fixed_fine_num_samples > 0:
        out['steps'] = out['steps'] * fixed_fine_num_samples
    if reduce_fine_for_missed:
        out['steps'] = out['steps'] * total
    if fine_num_sample_ratio > 0:
        out['steps'] = samples['sampled_point_voxel_idx'].ne(-1).sum(-1).float() * fine_num_sample_ratio
    return out


def render_rays(encoder, field, renderer, ray_start, ray_dir, encoder_states=None,
                fixed_num_samples=0, hierarchical=False, field_fine=None,
                fixed_fine_num_samples=0, fine_num_sample_ratio=0,
                reduce_fine_for_missed=False):
    """One frame of rays through the NSVF model glue: intersect, keep the hit
    rays, build the sampling distribution, sample, render, fill the missed
    rays with the background. ray_start [S, V, P, 3] (or [S, 1, 1, 3]
    broadcast), ray_dir [S, V, P, 3]; returns the reference's output dict
    (colors [S, V, P, 3], depths, missed, ...).
    hierarchical: a second, fine pass on samples placed by the coarse pass's
    probabilities (prepare_hierarchical_sampling), rendered with field_fine
    (or `field`); the coarse results are under 'coarse'
    (fairnr/models/fairnr_model.py:142-186)."""
    S, V, P, _ = ray_dir.size()
    if encoder_states is None:
        encoder_states = encoder.precompute(id=None)
    rs, rd, inter, hits = encoder.ray_intersect(ray_start, ray_dir, {
        k: (v.unsqueeze(0) if v is not None else None) for k, v in encoder_states.items()})
    # probs / steps (fairnr/models/nsvf.py:65-74), each ray's sum in slot
    # order (nsvf_ray_probs; the served chain's order too)
    inter['probs'], steps = ray_probs(inter['intersected_voxel_idx'], inter['min_depth'],
                                      inter['max_depth'], encoder.step_size)
    if fixed_num_samples > 0:
        inter['steps'] = inter['min_depth'].new_ones(*inter['min_depth'].size()[:-1], 1) * fixed_num_samples
    else:
        inter['steps'] = steps
    rs0, rd0 = rs.reshape(-1, 3), rd.reshape(-1, 3)
    all_results = defaultdict(lambda: None)
    coarse = None
    if hits.sum() > 0:
        sub = {name: outs[hits] for name, outs in inter.items()}
        rsh, rdh = rs[hits], rd[hits]
        samples = encoder.ray_sample(sub)
        all_results = renderer(encoder, field.forward, rsh, rdh, samples, encoder_states)
        all_results['voxel_depth'] = samples['sampled_point_depth'][:, 0]
        if hierarchical:
            sub = prepare_hierarchical_sampling(sub, samples, all_results, fixed_fine_num_samples,
                                                reduce_fine_for_missed, fine_num_sample_ratio)
            coarse = dict(all_results)
            samples = encoder.ray_sample(sub)
            fine = field_fine if field_fine is not None else field
            all_results = renderer(encoder, fine.forward, rsh, rdh, samples, encoder_states)
            all_results['voxel_depth'] = samples['sampled_point_depth'][:, 0]
    hits = hits.reshape(-1)
    out = _postprocess(all_results, hits, field, rs0, S, V, P)
    if coarse is not None:
        out['coarse'] = _postprocess(coarse, hits, field, rs0, S, V, P)
    return out


def _postprocess(all_results, hits, field, rs0, S, V, P):
    """fill_in + background (fairnr/models/nsvf.py:89-110)."""
    full = S * V * P
    out = dict(all_results)
    if all_results['missed'] is None:
        out['missed'] = rs0.new_ones(full)
        out['colors'] = rs0.new_zeros(full, 3)
        out['depths'] = rs0.new_zeros(full)
    out['missed'] = fill_in((full,), hits, out['missed'], 1.0).view(S, V, P)
    out['colors'] = fill_in((full, 3), hits, out['colors'], 0.0).view(S, V, P, 3)
    out['depths'] = fill_in((full,), hits, out['depths'], 0.0).view(S, V, P)
    bg = field.bg_color(out['colors'])
    out['colors'] = out['colors'] + out['missed'].unsqueeze(-1) * bg.reshape(full, 3).view(S, V, P, 3)
    out['depths'] = out['depths'] + out['missed'] * field.bg_color.depth
    return out
