"""Golden fixture of the training step (the differentiation workload), from
the reference's own autograd (run where the reference checkout is present):

    python tests/golden/make_golden_train.py

Workload: the 125,476-voxel c2 shell with N(0, 0.01^2) corner embeddings
(seed 1), the 4 x 128 field with its density row scaled 30x and bias 0.5 (an
opaque field, so that compositing gradients matter), a batch of 4 views
(cameras 0, 25, 50, 75 of the 100 on the radius-4 sphere, 800x800) x 2,048
pixels drawn (seed 21) among the pixels whose ray hits a voxel and enters no
two voxels at the same depth (where the reference's unstable depth sort is
free to order them either way), and targets
rendered from a second embedding set (seed 7). The rays themselves are stored
(their host computation is not bit-identical across CPU architectures:
numpy's matrix product rounds differently on Arm). Both sides sample with the
slot-order sampling distribution (oracle.cpu.probs_steps), so they evaluate
the same samples.

The reference side runs its SparseVoxelEncoder (bbox grid with the shell
kept, the embeddings placed by corner coordinates), its VolumeRenderer and a
field module with its field interface, on the CPU with autograd, and takes
loss = sum of squared colour errors (background white where rays miss the
rest of the way). Writes golden_train.npz: the pixel indices, the target
colours, the loss, every field-parameter gradient, and the embedding
gradient of 8,192 seeded corners among those the batch touches (by the
product encoder's corner ids, with their integer coordinates).
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
sys.path.insert(0, HERE)

from oracle import build_ref, cpu, ref_import, workload  # noqa: E402
from nsvf_gb300 import scenes  # noqa: E402
import make_golden as mg  # noqa: E402

VIEWS = (0, 25, 50, 75)
RAYS_PER_VIEW = 2048
SIGMA_SCALE, SIGMA_BIAS = 30.0, 0.5


def batch_pixels(sc):
    """(view, pixel) pairs: 2,048 hit pixels per view, seeded, among the rays
    that enter no two voxels at the same depth (for those the reference's
    unstable torch.sort may order the hits either way, and the samples with
    them)."""
    cen, chi = sc["octree"]
    rng = np.random.RandomState(21)
    out = []
    for v in VIEWS:
        rs, rd = workload.frame(v)
        idx, lo, _ = cpu.sort_hits(*cpu.svo_intersect(np.broadcast_to(rs, (rd.shape[0], 3))[None],
                                                      rd[None], cen[None], chi[None],
                                                      sc["voxel_size"], 64))
        idx, lo = idx[0], lo[0]
        tie = ((lo[:, 1:] == lo[:, :-1]) & (idx[:, 1:] != -1)).any(-1)
        hit = np.nonzero((idx != -1).any(-1) & ~tie)[0]
        out.append(np.sort(rng.choice(hit, RAYS_PER_VIEW, replace=False)))
    return np.stack(out)


def main():
    ref = ref_import.load()
    build_ref.build_clib()
    vs = 1.0 / 64
    sc = workload.c2_scene(vs)
    pix = batch_pixels(sc)
    rays_o, rays_d = [], []
    for v, p in zip(VIEWS, pix):
        rs, rd = workload.frame(v)
        rays_o.append(np.broadcast_to(rs, (p.size, 3)))
        rays_d.append(rd[p])
    rays_o = torch.from_numpy(np.concatenate(rays_o).astype(np.float32))
    rays_d = torch.from_numpy(np.concatenate(rays_d).astype(np.float32))
    R = rays_d.shape[0]

    # the reference encoder, embeddings placed by corner coordinates
    import make_golden_ops as mgo
    enc = mgo.c2_encoder(ref, sc["points"], vs)
    keys_prod, _ = workload.corner_table(sc["points"], vs)       # product corner ids
    ref_keys = enc.keys.numpy()
    # both are integer corner coordinates in half-voxel units, the
    # reference's relative to the bbox grid's first voxel (-1, -1, -1), the
    # product's to the shell's own minimum: shift by the difference
    hv = vs / 2
    p0 = sc["points"].astype(np.float64)
    shift = (np.round((p0[0] + 1.0) / hv) - np.round((p0[0] - p0.min(0)) / hv)).astype(np.int64)
    n = int(round(2.0 / hv)) + 3
    lin = lambda k: ((k.astype(np.int64) + 1) * np.array([n * n, n, 1])).sum(-1)
    ref_lin = lin(ref_keys)
    prod_lin = lin(keys_prod + shift)
    order = np.argsort(ref_lin)
    pos = order[np.searchsorted(ref_lin[order], prod_lin)]
    assert np.array_equal(ref_lin[pos], prod_lin)

    def set_values(seed):
        emb = scenes.voxel_embeddings(keys_prod.shape[0], 32, 0.01, seed=seed)
        with torch.no_grad():
            enc.values.weight.zero_()
            enc.values.weight[torch.from_numpy(pos)] = emb

    weights = scenes.stand_in_mlp_weights(seed=2, sigma_scale=SIGMA_SCALE, sigma_bias=SIGMA_BIAS)
    field = mg.StandInField(weights).eval()
    renderer = ref.renderer.VolumeRenderer(argparse.Namespace(chunk_size=64)).eval()
    st = enc.precompute(id=None)

    # samples: the reference's intersection and inverse-CDF placement on the
    # slot-order distribution
    _, _, out, hits = enc.ray_intersect(rays_o.reshape(1, 1, R, 3), rays_d.reshape(1, 1, R, 3),
                                        {k: (v.unsqueeze(0) if v is not None else None)
                                         for k, v in st.items()})
    h = hits.reshape(-1)
    assert bool(h.all())
    I = out["intersected_voxel_idx"].reshape(R, -1)
    L = out["min_depth"].reshape(R, -1)
    U = out["max_depth"].reshape(R, -1)
    pr, stp = cpu.probs_steps(I.numpy(), L.numpy(), U.numpy(), enc.step_size.item())
    sub = {"intersected_voxel_idx": I, "min_depth": L, "max_depth": U,
           "probs": torch.from_numpy(pr), "steps": torch.from_numpy(stp)}
    samples = enc.ray_sample(sub)

    def render():
        res = renderer(enc, field.forward, rays_o, rays_d, dict(samples), enc.precompute(id=None))
        return res["colors"] + res["missed"][:, None] * 1.0

    set_values(7)
    with torch.no_grad():
        target = render()
    set_values(1)
    enc.values.weight.grad = None
    field.zero_grad()
    colors = render()
    loss = ((colors - target) ** 2).sum()
    loss.backward()
    g = {"views": np.array(VIEWS), "pixels": pix, "ray_start": rays_o.numpy(),
         "ray_dir": rays_d.numpy(), "target": target.numpy(),
         "loss": np.float64(loss.item()), "sigma_scale": np.float32(SIGMA_SCALE),
         "sigma_bias": np.float32(SIGMA_BIAS),
         "n_samples": np.int64(int(samples["sampled_point_voxel_idx"].ne(-1).sum()))}
    for li, lin_ in enumerate(field.layers):
        g["grad_W%d" % li] = lin_.weight.grad.numpy()
        g["grad_b%d" % li] = lin_.bias.grad.numpy()
    gv = enc.values.weight.grad.numpy()[pos]            # in product corner order
    touched = np.nonzero(np.abs(gv).sum(-1) > 0)[0]
    sel = np.sort(np.random.RandomState(22).choice(touched, min(8192, touched.size), replace=False))
    g["grad_values_keys"] = sel.astype(np.int64)
    g["grad_values_rows"] = gv[sel]
    g["grad_values_norm"] = np.float64(np.sqrt((gv.astype(np.float64) ** 2).sum()))
    g["grad_values_touched"] = np.int64(touched.size)
    np.savez_compressed(os.path.join(HERE, "golden_train.npz"), **g)
    print("wrote golden_train.npz: %d rays, %d samples, loss %.6g, %d corners touched"
          % (R, g["n_samples"], loss.item(), touched.size))


if __name__ == "__main__":
    main()
