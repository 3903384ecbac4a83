"""Generate the golden fixtures in tests/golden/ from the reference itself.

Run in the container that holds the reference checkout:

    python tests/golden/make_golden.py

It imports the reference's pure-PyTorch modules (SparseVoxelEncoder,
VolumeRenderer, geometry) through oracle/ref_import.py, whose fairnr.clib._ext
stand-in runs the reference's own kernel bodies and octree builder compiled
for the CPU (oracle/build_ref.py). The field is the workloads' stand-in MLP
(32 -> 4 x 128 ReLU -> sigma, rgb) written here as a small torch module with
the reference field interface.

Fixtures (npz, compressed), all on the 147-voxel "small" scene (voxel 0.25,
64x64 view, focal 80, max_hits 20, step voxel/8):

* golden_small.npz -- scene, octree, rays (a 1024-ray subset), raw AABB and
  SVO op outputs, the encoder's sorted intersection, probs/steps, the
  inverse-CDF samples for deterministic and for recorded seeded noise,
  embeddings at the samples, and the rendered colors/depths/missed/probs.
* golden_prune.npz -- pruning masks: the reference rule (16^3 points,
  keep = 1 - min exp(-relu sigma) > 0.5) and the workload rule
  (8^3 points, keep = max(1 - exp(-relu(sigma) * step)) >= th, th = 0.3 here).
"""
import argparse
import os
import sys
import tempfile

import numpy as np
import torch
import torch.nn as nn

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import ref_import, build_ref  # noqa: E402
from nsvf_gb300 import scenes  # noqa: E402


# density scale of the golden field: opaque enough that compositing and both
# pruning rules see a mix of empty and occupied voxels
GOLDEN_SIGMA_SCALE = 60.0
GOLDEN_SIGMA_BIAS = 0.5
# threshold of the sigma*step rule on this small scene (0.5 in the 125k-voxel
# workload); 0.3 splits the 147 voxels into kept and pruned ones
PRUNE8_TH = 0.3


class StandInField(nn.Module):
    """4 x 128 ReLU MLP on the 32-d embedding -> (sigma, rgb), with the
    reference field's call convention: forward(inputs, outputs) -> inputs."""

    def __init__(self, weights):
        super().__init__()
        self.layers = nn.ModuleList()
        for W, b in weights:
            lin = nn.Linear(W.shape[1], W.shape[0])
            lin.weight.data.copy_(W)
            lin.bias.data.copy_(b)
            self.layers.append(lin)

    def forward(self, inputs, outputs=("sigma", "texture")):
        x = inputs["emb"]
        for i, lin in enumerate(self.layers):
            x = lin(x)
            if i < len(self.layers) - 1:
                x = torch.relu(x)
        inputs["sigma"] = x[:, 0]
        if "texture" in outputs:
            inputs["texture"] = x[:, 1:4]
        return inputs


def make_encoder(ref, points, voxel_size, use_octree, embed):
    """The reference encoder on the bbox [-1, 1]^3 grid with the voxels outside
    `points` pruned through its `keep` buffer (the reference's .txt voxel
    files leave voxel_size unset, fairnr/modules/encoder.py:246-249)."""
    path = tempfile.mktemp(suffix=".txt")
    np.savetxt(path, np.array([[-1, -1, -1, 1, 1, 1, voxel_size]]))
    args = argparse.Namespace(voxel_path=None, initial_boundingbox=path, voxel_size=voxel_size,
                              max_hits=20, raymarching_stepsize_ratio=0.125, voxel_embed_dim=32,
                              use_octree=use_octree, deterministic_step=True)
    enc = ref.encoder.SparseVoxelEncoder(args)
    os.unlink(path)
    allp = enc.points.numpy()
    keep = (allp[:, None, :] == points[None]).all(-1).any(-1)
    assert keep.sum() == points.shape[0]
    assert np.array_equal(allp[keep], points)
    enc.keep.copy_(torch.from_numpy(keep).long())
    enc.values.weight.data.copy_(embed[: enc.values.weight.shape[0]])
    enc.eval()
    return enc


def probs_steps(out, step_size):
    # fairnr/models/nsvf.py:65-74
    d = (out["max_depth"] - out["min_depth"]).masked_fill(out["intersected_voxel_idx"].eq(-1), 0)
    out["probs"] = d / d.sum(dim=-1, keepdim=True)
    out["steps"] = d.sum(-1) / step_size
    return out


def main():
    ref = ref_import.load()
    build_ref.build_clib()
    torch.manual_seed(0)
    pts, vs = scenes.scene_small()
    rs, rd = scenes.small_view(0)
    embed = scenes.voxel_embeddings(1000, 32, std=1.0, seed=1)
    weights = scenes.stand_in_mlp_weights(seed=2, sigma_scale=GOLDEN_SIGMA_SCALE,
                                          sigma_bias=GOLDEN_SIGMA_BIAS)
    field = StandInField(weights).eval()
    g = {}
    g["points"] = pts
    g["voxel_size"] = np.float32(vs)
    g["embed"] = embed.numpy()
    for li, (W, b) in enumerate(weights):
        g["W%d" % li] = W.numpy()
        g["b%d" % li] = b.numpy()

    sel = np.arange(0, rd.shape[0], 4)              # 1024-ray subset, every 4th pixel
    ray_dir = torch.from_numpy(rd[sel]).reshape(1, 1, -1, 3)
    ray_start = torch.from_numpy(rs).reshape(1, 1, 1, 3)
    g["ray_start"] = rs
    g["ray_dir"] = rd[sel]

    for use_octree, tag in [(False, "aabb"), (True, "svo")]:
        enc = make_encoder(ref, pts, vs, use_octree, embed)
        st = enc.precompute(id=None)
        if use_octree:
            g["octree_centers"] = st["voxel_octree_center_xyz"].numpy()
            g["octree_children"] = st["voxel_octree_children_idx"].numpy()
        g["%s_centers_shifted" % tag] = st["voxel_center_xyz"].numpy()
        g["feats"] = st["voxel_vertex_idx"].numpy()
        g["keep"] = enc.keep.numpy()
        g["num_keys"] = np.int64(enc.num_keys)
        # raw op outputs
        R = ray_dir.shape[2]
        rs3 = ray_start.expand(1, 1, R, 3).reshape(1, R, 3).contiguous()
        rd3 = ray_dir.reshape(1, R, 3).contiguous()
        if use_octree:
            raw = ref.clib.svo_ray_intersect(vs, 20, st["voxel_octree_center_xyz"].unsqueeze(0),
                                             st["voxel_octree_children_idx"].unsqueeze(0), rs3, rd3)
        else:
            raw = ref.clib.aabb_ray_intersect(vs, 20, st["voxel_center_xyz"].unsqueeze(0), rs3, rd3)
        for k, v in zip(["idx", "min", "max"], raw):
            g["%s_raw_%s" % (tag, k)] = v.numpy()
        # encoder post-processing
        _, _, out, hits = enc.ray_intersect(ray_start, ray_dir, {
            k: (v.unsqueeze(0) if v is not None else None) for k, v in st.items()})
        out = probs_steps(out, enc.step_size)
        for k in ["intersected_voxel_idx", "min_depth", "max_depth", "probs", "steps"]:
            g["%s_%s" % (tag, k)] = out[k].numpy()
        g["%s_hits" % tag] = hits.numpy()
        if not use_octree:
            continue
        # sampling on the hit rays: deterministic, then seeded noise (recorded)
        h = hits.reshape(-1)
        sub = {k: v.reshape(-1, v.shape[-1])[h] if v.dim() == 3 else v.reshape(-1)[h]
               for k, v in out.items()}
        samples = enc.ray_sample(sub)
        for k, v in samples.items():
            g["svo_det_%s" % k] = v.numpy()
        gen_state = torch.get_rng_state()
        enc.train()
        enc.deterministic_step = False
        torch.manual_seed(123)
        samples_rand = enc.ray_sample(sub)
        torch.manual_seed(123)
        N, P = sub["intersected_voxel_idx"].shape
        Hp = int(np.ceil(N / 200)) * 200
        M = int(sub["steps"].ceil().long().max()) + P
        noise = torch.zeros(Hp, M).uniform_().clamp(min=0.001, max=0.999)
        torch.set_rng_state(gen_state)
        enc.eval()
        enc.deterministic_step = True
        g["svo_noise"] = noise.numpy()
        for k, v in samples_rand.items():
            g["svo_rand_%s" % k] = v.numpy()
        # embeddings and rendering on the deterministic samples
        rsh = ray_start.reshape(1, 3).expand(N, 3)
        rdh = ray_dir.reshape(-1, 3)[h]
        sampled_xyz = rsh.unsqueeze(1) + rdh.unsqueeze(1) * samples["sampled_point_depth"].unsqueeze(2)
        mask = samples["sampled_point_voxel_idx"].ne(-1)
        emb_in = {"sampled_point_xyz": sampled_xyz[mask],
                  "sampled_point_voxel_idx": samples["sampled_point_voxel_idx"][mask],
                  "sampled_point_ray_direction": rdh.unsqueeze(1).expand_as(sampled_xyz)[mask],
                  "sampled_point_distance": samples["sampled_point_distance"][mask]}
        emb = enc.forward(emb_in, st)["emb"]
        g["svo_det_emb"] = emb.detach().numpy()[:2048]
        renderer = ref.renderer.VolumeRenderer(argparse.Namespace(chunk_size=64)).eval()
        with torch.no_grad():
            res = renderer(enc, field, rsh, rdh, dict(samples), st)
        for k in ["colors", "depths", "missed", "probs"]:
            g["render_%s" % k] = res[k].detach().numpy()
        # training step gradients (reference autograd): loss against a target
        # rendered from a second seeded embedding set
        embed2 = scenes.voxel_embeddings(1000, 32, std=1.0, seed=7)
        enc2 = make_encoder(ref, pts, vs, True, embed2)
        st2 = enc2.precompute(id=None)
        with torch.no_grad():
            tgt = renderer(enc2, field, rsh, rdh, dict(samples), st2)["colors"]
        enc.values.weight.grad = None
        field.zero_grad()
        st_g = enc.precompute(id=None)
        res_g = renderer(enc, field, rsh, rdh, dict(samples), st_g)
        loss = ((res_g["colors"] - tgt) ** 2).sum()
        loss.backward()
        g["grad_target_colors"] = tgt.numpy()
        g["grad_loss"] = np.float64(loss.item())
        g["grad_values"] = enc.values.weight.grad.numpy()
        g["grad_W0"] = field.layers[0].weight.grad.numpy()
        g["grad_W4"] = field.layers[4].weight.grad.numpy()

    np.savez_compressed(os.path.join(HERE, "golden_small.npz"), **g)

    # pruning: reference rule (bits 16) and the workload rule (bits 8, sigma * step)
    enc = make_encoder(ref, pts, vs, True, embed)
    st = enc.precompute(id=None)
    with torch.no_grad():
        sc16 = enc.get_scores(field.forward, th=0.5, bits=16, encoder_states=st)
        keep16 = (1 - sc16.min(-1)[0]) > 0.5
        # workload rule: sigma at 8^3 points per voxel through the reference's
        # own point generation and embedding (the body of get_scores_once,
        # fairnr/modules/encoder.py:629-651, without its exp)
        pts8 = ref.geometry.offset_points(st["voxel_center_xyz"], enc.voxel_size / 2.0, bits=8)
        idx8 = torch.arange(pts8.size(0))[:, None].expand(*pts8.size()[:2])
        emb8 = enc.forward({"sampled_point_xyz": pts8.reshape(-1, 3),
                            "sampled_point_voxel_idx": idx8.reshape(-1),
                            "sampled_point_ray_direction": None,
                            "sampled_point_distance": None}, st)
        sigma8 = field.forward(emb8, outputs=["sigma"])["sigma"].reshape(-1, 512)
        step = float(enc.step_size)
        alpha8 = 1 - torch.exp(-torch.relu(sigma8) * step)
        keep8 = alpha8.max(-1)[0] >= PRUNE8_TH
    np.savez_compressed(os.path.join(HERE, "golden_prune.npz"),
                        keep16=keep16.numpy(), keep8=keep8.numpy(),
                        minscore16=sc16.min(-1)[0].numpy(), maxalpha8=alpha8.max(-1)[0].numpy(),
                        step=np.float32(step), th8=np.float32(PRUNE8_TH))
    print("pruning: keep16 %d/%d, keep8 %d/%d" % (int(keep16.sum()), keep16.numel(),
                                                  int(keep8.sum()), keep8.numel()))
    print("wrote golden fixtures", {k: getattr(v, "shape", None) for k, v in g.items()})


if __name__ == "__main__":
    main()
