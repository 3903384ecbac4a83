"""Drop-in SparseVoxelEncoder (fairnr/modules/encoder.py:202-712).

Same constructor, buffers (points, keys, feats, num_keys, keep, voxel_size,
step_size, max_hits; fairnr/modules/encoder.py:285-293), `values` embedding
and methods. The hot methods run on the sm_103a kernels:

* ray_intersect: the octree's sorted hit lists from the leaf-grid sweep
  (nsvf_svo_intersect_grid, one octree), or the SVO traversal with the depth
  sort fused into the kernel (nsvf_svo_intersect_sorted), or the brute-force
  AABB kernel + sort;
* ray_sample:    inverse-CDF sampling kernel (nsvf_gb300.clib);
* forward:       trilinear interpolation kernel with a hand-written backward;
* octree build:  native host builder (about 150x faster than the reference's
                 at::Tensor-per-element build on the 125k-voxel scene).

Voxel files: the reference's .txt format (columns 3:6 = centres) needs
args.voxel_size (the reference leaves it unset on that path); .ply needs the
optional plyfile package.
"""
import logging
import os

import numpy as np
import torch
import torch.distributed as dist
import torch.nn as nn
import torch.nn.functional as F

from . import clib, ext
from .functional import trilinear_embed
from .geometry import (bbox2voxels, build_easy_octree, discretize_points, offset_points,
                       splitting_points, voxel_corner_table)

logger = logging.getLogger(__name__)
MAX_DEPTH = 10000.0


def Embedding(num_embeddings, embedding_dim, padding_idx=None):
    m = nn.Embedding(num_embeddings, embedding_dim, padding_idx=padding_idx)
    nn.init.normal_(m.weight, mean=0, std=embedding_dim ** -0.5)
    return m


class SparseVoxelEncoder(nn.Module):

    def __init__(self, args, voxel_path=None, bbox_path=None, shared_values=None, points=None):
        super().__init__()
        self.args = args
        self.voxel_path = voxel_path if voxel_path is not None else getattr(args, "voxel_path", None)
        self.bbox_path = bbox_path if bbox_path is not None else getattr(args, "initial_boundingbox", None)
        self.voxel_index = None
        self.scene_scale = getattr(args, "scene_scale", 1.0)
        if points is not None:                      # voxel centres given directly
            fine_points = torch.as_tensor(points, dtype=torch.float32)
            voxel_size = args.voxel_size
        elif self.voxel_path is not None:
            if not os.path.exists(self.voxel_path):
                raise FileNotFoundError(self.voxel_path)
            if self.voxel_path.endswith(".ply"):
                from plyfile import PlyData   # optional dependency
                ply = PlyData.read(self.voxel_path)
                v = ply["vertex"]
                fine_points = torch.from_numpy(np.stack([v["x"], v["y"], v["z"]]).astype("float32").T)
                voxel_size = args.voxel_size
                if "quality" in [p.name for p in v.properties]:
                    self.voxel_index = torch.from_numpy(v["quality"]).long()
            else:
                fine_points = torch.from_numpy(np.loadtxt(self.voxel_path)[:, 3:].astype("float32"))
                voxel_size = args.voxel_size
        elif self.bbox_path is not None:
            bbox = np.loadtxt(self.bbox_path)
            voxel_size = bbox[-1] if getattr(args, "voxel_size", None) is None else args.voxel_size
            fine_points = torch.from_numpy(bbox2voxels(bbox[:6], voxel_size))
        else:
            raise ValueError("at least initial bounding box or pretrained voxel files are required.")

        fine_keys, fine_feats = voxel_corner_table(fine_points, voxel_size)
        num_keys = torch.scalar_tensor(fine_keys.size(0)).long()
        if getattr(args, "raymarching_stepsize_ratio", 0) > 0:
            step_size = args.raymarching_stepsize_ratio * voxel_size
        else:
            step_size = args.raymarching_stepsize

        self.register_buffer("points", fine_points)
        self.register_buffer("keys", fine_keys.long())
        self.register_buffer("feats", fine_feats.long())
        self.register_buffer("num_keys", num_keys)
        self.register_buffer("keep", fine_feats.new_ones(fine_feats.size(0)).long())
        self.register_buffer("voxel_size", torch.scalar_tensor(voxel_size))
        self.register_buffer("step_size", torch.scalar_tensor(step_size))
        self.register_buffer("max_hits", torch.scalar_tensor(args.max_hits))

        self.embed_dim = getattr(args, "voxel_embed_dim", None)
        self.deterministic_step = getattr(args, "deterministic_step", False)
        self.use_octree = getattr(args, "use_octree", False)
        self.track_max_probs = getattr(args, "track_max_probs", False)
        self._runtime_caches = {"flatten_centers": None, "flatten_children": None,
                                "max_voxel_probs": None, "svo_grid": None}
        if shared_values is None and self.embed_dim and self.embed_dim > 0:
            self.values = Embedding(int(num_keys), self.embed_dim, None)
        else:
            self.values = shared_values

    # ------------------------------------------------------------ state --
    def upgrade_state_dict_named(self, state_dict, name):
        if self.values is not None:
            loaded = state_dict[name + '.values.weight']
            self.values.weight = nn.Parameter(self.values.weight.new_zeros(*loaded.size()))
            self.values.num_embeddings = self.values.weight.size(0)
            self.total_size = self.values.weight.size(0)
            self.num_keys = self.num_keys * 0 + self.total_size
        if self.voxel_index is not None:
            for k in ("points", "feats", "keep"):
                state_dict[name + '.' + k] = state_dict[name + '.' + k][self.voxel_index]
        if name + '.points' in state_dict:
            self.points = self.points.new_zeros(*state_dict[name + '.points'].size())
            self.feats = self.feats.new_zeros(*state_dict[name + '.feats'].size())
            self.keys = self.keys.new_zeros(*state_dict[name + '.keys'].size())
            self.keep = self.keep.new_zeros(*state_dict[name + '.keep'].size())
        else:
            for k in ("points", "feats", "keys", "keep", "voxel_size", "step_size", "max_hits",
                      "num_keys"):
                state_dict[name + '.' + k] = getattr(self, k)

    @staticmethod
    def add_args(parser):
        parser.add_argument('--initial-boundingbox', type=str)
        parser.add_argument('--voxel-size', type=float, metavar='D')
        parser.add_argument('--voxel-path', type=str)
        parser.add_argument('--voxel-embed-dim', type=int, metavar='N')
        parser.add_argument('--deterministic-step', action='store_true')
        parser.add_argument('--max-hits', type=int, metavar='N')
        parser.add_argument('--raymarching-stepsize', type=float, metavar='D')
        parser.add_argument('--raymarching-stepsize-ratio', type=float, metavar='D')
        parser.add_argument('--use-octree', action='store_true')
        parser.add_argument('--track-max-probs', action='store_true')
        parser.add_argument('--scene-scale', type=float, default=1.0)

    # ----------------------------------------------------------- caches --
    def reset_runtime_caches(self):
        if self.use_octree:
            points = self.points[self.keep.bool()]
            centers, children = build_easy_octree(points, self.voxel_size / 2.0)
            self._runtime_caches['flatten_centers'] = centers
            self._runtime_caches['flatten_children'] = children
            self._runtime_caches['svo_grid'] = None
        if self.track_max_probs:
            self._runtime_caches['max_voxel_probs'] = self.points.new_zeros(self.points.size(0))

    def clean_runtime_caches(self):
        for name in self._runtime_caches:
            self._runtime_caches[name] = None

    @property
    def flatten_centers(self):
        if self._runtime_caches['flatten_centers'] is None:
            self.reset_runtime_caches()
        return self._runtime_caches['flatten_centers']

    @property
    def flatten_children(self):
        if self._runtime_caches['flatten_children'] is None:
            self.reset_runtime_caches()
        return self._runtime_caches['flatten_children']

    def svo_grid(self, centers, children):
        """The leaf-grid form (ext.SvoGrid) of the octree `centers` [N, 3],
        `children` [N, 9] of this encoder's states, built once per octree on
        the first intersection and kept with the runtime caches; None when
        the states' octree is not this encoder's (checked by value) or not in
        leaf-grid form."""
        fc, fch = self.flatten_centers, self.flatten_children
        if fc is None or centers.shape != fc.shape or children.shape != fch.shape:
            return None
        g = self._runtime_caches.get('svo_grid')
        if g is None or g.centers.device != centers.device:
            g = ext.SvoGrid(fc.to(centers.device).float().contiguous(),
                            fch.to(centers.device).int().contiguous(), float(self.voxel_size))
            self._runtime_caches['svo_grid'] = g
        if not g.ok or g.voxel_size != float(self.voxel_size):
            return None
        if not (torch.equal(centers, g.centers) and torch.equal(children, g.children)):
            return None
        return g

    @property
    def max_voxel_probs(self):
        if self._runtime_caches['max_voxel_probs'] is None:
            self.reset_runtime_caches()
        return self._runtime_caches['max_voxel_probs']

    @max_voxel_probs.setter
    def max_voxel_probs(self, x):
        self._runtime_caches['max_voxel_probs'] = x

    # ------------------------------------------------------- precompute --
    def precompute(self, id=None, *args, **kwargs):
        feats = self.feats[self.keep.bool()]
        points = self.points[self.keep.bool()]
        points[:, 0] += (self.voxel_size / 10)      # the reference's x shift (encoder.py:383)
        values = self.values.weight[: self.num_keys] if self.values is not None else None
        if id is not None:
            feats = feats.unsqueeze(0).expand(id.size(0), *feats.size()).contiguous()
            points = points.unsqueeze(0).expand(id.size(0), *points.size()).contiguous()
            values = values.unsqueeze(0).expand(id.size(0), *values.size()).contiguous() \
                if values is not None else None
            if id.size(0) > 1:
                feats = feats + self.num_keys * torch.arange(
                    id.size(0), device=feats.device, dtype=feats.dtype)[:, None, None]
        states = {'voxel_vertex_idx': feats, 'voxel_center_xyz': points, 'voxel_vertex_emb': values}
        if self.use_octree:
            c, ch = self.flatten_centers.clone(), self.flatten_children.clone()
            if id is not None:
                c = c.unsqueeze(0).expand(id.size(0), *c.size()).contiguous()
                ch = ch.unsqueeze(0).expand(id.size(0), *ch.size()).contiguous()
            states['voxel_octree_center_xyz'] = c
            states['voxel_octree_children_idx'] = ch
        return states

    # -------------------------------------------------------- intersect --
    def ray_intersect(self, ray_start, ray_dir, encoder_states):
        point_feats = encoder_states['voxel_vertex_idx']
        point_xyz = encoder_states['voxel_center_xyz']
        S, V, P, _ = ray_dir.size()
        _, H, D = point_feats.size()
        ray_start = ray_start.expand_as(ray_dir).contiguous().view(S, V * P, 3).contiguous()
        ray_dir = ray_dir.reshape(S, V * P, 3).contiguous()
        n_max = int(self.max_hits)
        grid = None
        if self.use_octree and n_max <= 128 and ray_start.dtype == torch.float32:
            oc = encoder_states['voxel_octree_center_xyz'].float().contiguous()
            och = encoder_states['voxel_octree_children_idx'].int().contiguous()
            if S == 1 and oc.dim() == 3 and ray_start.is_cuda:
                grid = self.svo_grid(oc[0], och[0])
        if grid is not None:
            # the leaf-grid sweep: the same sorted lists as the traversal + sort
            pts_idx, min_depth, max_depth, hits = ext.svo_intersect_grid(
                grid, ray_start, ray_dir, n_max)
        elif self.use_octree and n_max <= 128 and ray_start.dtype == torch.float32:
            pts_idx, min_depth, max_depth, hits = ext.svo_intersect_sorted(
                ray_start, ray_dir, oc, och, float(self.voxel_size), n_max)
        else:
            if self.use_octree:
                pts_idx, min_depth, max_depth = clib.svo_ray_intersect(
                    self.voxel_size, n_max, encoder_states['voxel_octree_center_xyz'],
                    encoder_states['voxel_octree_children_idx'], ray_start, ray_dir)
            else:
                pts_idx, min_depth, max_depth = clib.aabb_ray_intersect(
                    self.voxel_size, n_max, point_xyz, ray_start, ray_dir)
            min_depth.masked_fill_(pts_idx.eq(-1), MAX_DEPTH)
            max_depth.masked_fill_(pts_idx.eq(-1), MAX_DEPTH)
            min_depth, sorted_idx = min_depth.sort(dim=-1, stable=True)
            max_depth = max_depth.gather(-1, sorted_idx)
            pts_idx = pts_idx.gather(-1, sorted_idx)
            hits = pts_idx.ne(-1).any(-1)
        if S > 1:
            pts_idx = (pts_idx + H * torch.arange(S, device=pts_idx.device, dtype=pts_idx.dtype)[:, None, None]
                       ).masked_fill_(pts_idx.eq(-1), -1)
        return ray_start, ray_dir, {"min_depth": min_depth, "max_depth": max_depth,
                                    "intersected_voxel_idx": pts_idx}, hits

    def ray_sample(self, intersection_outputs):
        sampled_idx, sampled_depth, sampled_dists = clib.inverse_cdf_sampling(
            intersection_outputs['intersected_voxel_idx'], intersection_outputs['min_depth'],
            intersection_outputs['max_depth'], intersection_outputs['probs'],
            intersection_outputs['steps'], -1, self.deterministic_step or (not self.training))
        sampled_dists = sampled_dists.clamp(min=0.0)
        sampled_depth = sampled_depth.masked_fill(sampled_idx.eq(-1), MAX_DEPTH)
        sampled_dists = sampled_dists.masked_fill(sampled_idx.eq(-1), 0.0)
        return {'sampled_point_depth': sampled_depth, 'sampled_point_distance': sampled_dists,
                'sampled_point_voxel_idx': sampled_idx}

    @torch.enable_grad()
    def forward(self, samples, encoder_states):
        point_feats = encoder_states['voxel_vertex_idx']
        point_xyz = encoder_states['voxel_center_xyz']
        values = encoder_states['voxel_vertex_emb']
        sampled_idx = samples['sampled_point_voxel_idx'].long()
        sampled_xyz = samples['sampled_point_xyz'].requires_grad_(True)
        inputs = {'pos': sampled_xyz, 'ray': samples['sampled_point_ray_direction'],
                  'dists': samples['sampled_point_distance']}
        if values is not None:
            inputs['emb'] = trilinear_embed(sampled_idx, sampled_xyz,
                                            point_xyz.reshape(-1, 3), point_feats.reshape(-1, 8),
                                            values.reshape(-1, values.size(-1)),
                                            float(self.voxel_size))
        return inputs

    @torch.no_grad()
    def track_voxel_probs(self, voxel_idxs, voxel_probs):
        voxel_idxs = voxel_idxs.masked_fill(voxel_idxs.eq(-1), self.max_voxel_probs.size(0))
        chunk_size = 4096
        for start in range(0, voxel_idxs.size(0), chunk_size):
            end = min(start + chunk_size, voxel_idxs.size(0))
            m = self.max_voxel_probs.new_zeros(end - start, self.max_voxel_probs.size(0) + 1).scatter_add_(
                dim=-1, index=voxel_idxs[start:end], src=voxel_probs[start:end]).max(0)[0][:-1].data
            self.max_voxel_probs = torch.max(self.max_voxel_probs, m)

    # ---------------------------------------------------------- pruning --
    @torch.no_grad()
    def pruning(self, field_fn, th=0.5, encoder_states=None, train_stats=False, bits=16,
                use_step=False):
        """The reference's pruning (fairnr/modules/encoder.py:605-618) with the
        field in FP32: keep = 1 - min exp(-relu sigma) > th over bits^3 points
        per voxel (bits 16 as the reference). use_step selects the sigma * step
        rule: keep = max 1 - exp(-relu(sigma) * step) >= th (the c2 workload
        uses it with bits 8)."""
        if not train_stats:
            scores = self.get_scores(field_fn, th=th, bits=bits, encoder_states=encoder_states,
                                     use_step=use_step)
            keep = scores.max(-1)[0] >= th if use_step else (1 - scores.min(-1)[0]) > th
        else:
            if dist.is_initialized() and dist.get_world_size() > 1:
                dist.all_reduce(self.max_voxel_probs, op=dist.ReduceOp.MAX)
            keep = self.max_voxel_probs > th
        self.keep.masked_scatter_(self.keep.bool(), keep.long())
        logger.info("pruning done. # of voxels before: %d, after: %d", keep.size(0), int(keep.sum()))

    def get_scores(self, field_fn, th=0.5, bits=16, encoder_states=None, chunk_size=64,
                   use_step=False):
        """exp(-relu(sigma)) at bits^3 points per voxel: [V, bits^3]
        (fairnr/modules/encoder.py:620-654); with use_step the alphas
        1 - exp(-relu(sigma) * step) instead."""
        if encoder_states is None:
            encoder_states = self.precompute(id=None)
        feats = encoder_states['voxel_vertex_idx']
        points = encoder_states['voxel_center_xyz']
        values = encoder_states['voxel_vertex_emb']

        def once(feats, points):
            xyz = offset_points(points, self.voxel_size / 2.0, bits=bits)
            idx = torch.arange(points.size(0), device=points.device)[:, None].expand(*xyz.size()[:2])
            inputs = self.forward({'sampled_point_xyz': xyz.reshape(-1, 3),
                                   'sampled_point_voxel_idx': idx.reshape(-1),
                                   'sampled_point_ray_direction': None,
                                   'sampled_point_distance': None},
                                  {'voxel_vertex_idx': feats, 'voxel_center_xyz': points,
                                   'voxel_vertex_emb': values})
            if encoder_states.get('context', None) is not None:
                inputs['context'] = encoder_states['context']
            out = field_fn(inputs, outputs=['sigma'])
            if use_step:
                return 1 - torch.exp(-torch.relu(out['sigma']).reshape(-1, bits ** 3) * self.step_size)
            return torch.exp(-torch.relu(out['sigma']).reshape(-1, bits ** 3))

        return torch.cat([once(feats[i:i + chunk_size], points[i:i + chunk_size])
                          for i in range(0, points.size(0), chunk_size)], 0)

    @torch.no_grad()
    def pruning_exact(self, mlp, th=0.5, bits=16, use_step=False, apply=True):
        """pruning() on the GPU with the mask decided exactly: the tensor-core
        BF16 pass screens every point and the points it cannot decide are
        evaluated in double-float (TensorCoreMLP.prune_mask). The mask is the
        reference rule's without rounding error. Returns the keep mask over
        the currently kept voxels (applied to `keep` unless apply=False)."""
        states = self.precompute(id=None)
        centers = states['voxel_center_xyz'].float().contiguous()
        feats = states['voxel_vertex_idx'].int().contiguous()
        values = states['voxel_vertex_emb'].detach().float().contiguous()
        keep, _, n = mlp.prune_mask(centers, feats, values, float(self.voxel_size), th=th,
                                    bits=bits, rule=1 if use_step else 0,
                                    step=float(self.step_size))
        self.last_prune_undecided_points = n
        if apply:
            self.keep.masked_scatter_(self.keep.bool(), keep.long())
            self.clean_runtime_caches()
        return keep

    @torch.no_grad()
    def pruning_fused(self, mlp, th=0.5, bits=8, rule=1, apply=True):
        """Self-pruning in one tensor-core kernel (nsvf_prune_scores_bf16):
        sigma at bits^3 points per voxel with the BF16 field. rule 0 is the
        reference's (keep = 1 - min exp(-relu sigma) > th, bits 16 there);
        rule 1 keeps voxels with max(1 - exp(-relu(sigma) * step)) >= th.
        Returns the keep mask over the currently kept voxels."""
        states = self.precompute(id=None)
        centers = states['voxel_center_xyz'].float().contiguous()
        feats = states['voxel_vertex_idx'].int().contiguous()
        values = states['voxel_vertex_emb'].detach().float().contiguous()
        score = mlp.prune_scores(centers, feats, values, float(self.voxel_size), bits=bits,
                                 rule=rule, step=float(self.step_size))
        keep = ((1 - score) > th) if rule == 0 else (score >= th)
        if apply:
            self.keep.masked_scatter_(self.keep.bool(), keep.long())
            self.clean_runtime_caches()
        return keep

    @torch.no_grad()
    def splitting(self):
        states = self.precompute(id=None)
        feats, points, values = states['voxel_vertex_idx'], states['voxel_center_xyz'], states['voxel_vertex_emb']
        new_points, new_feats, new_values, new_keys = splitting_points(points, feats, values,
                                                                      self.voxel_size / 2.0)
        if new_values is not None:
            self.values.weight = nn.Parameter(new_values)
            self.values.num_embeddings = self.values.weight.size(0)
        self.total_size = new_keys.size(0)
        self.num_keys = self.num_keys * 0 + self.total_size
        self.points = new_points
        self.feats = new_feats
        self.keep = self.keep.new_ones(new_points.size(0))

    @property
    def feature_dim(self):
        return self.embed_dim

    @property
    def dummy_loss(self):
        if self.values is not None:
            return self.values.weight[0, 0] * 0.0
        return 0.0

    @property
    def num_voxels(self):
        return self.keep.long().sum()
