"""Golden fixtures for the ops the small-scene fixtures leave out, from the
reference itself (run where the reference checkout is present):

    python tests/golden/make_golden_ops.py

It runs the reference's own fairnr.clib wrappers, encoder and geometry through
oracle/ref_import.py (the reference's kernel bodies compiled for the CPU,
oracle/build_ref.py). Writes golden_ops.npz:

* par_* -- the back-up parallel uniform sampler (`_parallel_ray_sampling`,
  fairnr/clib/__init__.py:303-349) on the 147-voxel scene's sorted hit lists
  (golden_small.npz) at step voxel/8: deterministic, and with torch seed 5
  (its [rays, steps] jitter recorded as par_noise);
* uni_* -- the UniformRaySampling op wrapper (fairnr/clib/__init__.py:
  176-226) on the same lists, max_ray_length 4: deterministic, and with
  torch seed 6 (its [256, rays/256, steps] noise recorded as uni_noise);
* ball_* -- ball_intersect (fairnr/clib/src/intersect_gpu.cu:15-70) of the
  1,024 golden rays against the 147 voxel centres, radius 0.15, n_max 20;
* c2_* -- 6,000 seeded rays from the central 400x400 pixels of the 800x800
  c2 frame 0 (125,476-voxel shell, max_hits 64, step 1/512): the raw SVO op
  outputs (the reference kernel on one octree copy), the encoder's sorted
  lists and hit flags, probs/steps (fairnr/models/nsvf.py:65-74), the
  deterministic inverse-CDF samples of the hit rays (the reference wrapper,
  200 blocks), and the parallel sampler on the hit rays (two 4,096-ray
  chunks, deterministic).
"""
import argparse
import os
import sys
import tempfile

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref, ref_import  # noqa: E402
from nsvf_gb300 import scenes  # noqa: E402


def c2_encoder(ref, points, vs):
    """The reference encoder on the [-1, 1]^3 bbox grid at voxel `vs` with the
    voxels outside `points` pruned through its `keep` buffer (its .txt voxel
    files leave voxel_size unset, fairnr/modules/encoder.py:246-249). Grid
    voxels are matched to `points` by integer grid coordinates."""
    path = tempfile.mktemp(suffix=".txt")
    np.savetxt(path, np.array([[-1, -1, -1, 1, 1, 1, vs]]))
    args = argparse.Namespace(voxel_path=None, initial_boundingbox=path, voxel_size=vs,
                              max_hits=64, raymarching_stepsize_ratio=0.125, voxel_embed_dim=32,
                              use_octree=True, deterministic_step=True)
    enc = ref.encoder.SparseVoxelEncoder(args)
    os.unlink(path)
    allp = enc.points.numpy()
    n = int(round(2.0 / vs)) + 1
    lin = lambda q: (np.round((q.astype(np.float64) + 1.0) / vs).astype(np.int64) *
                     np.array([n * n, n, 1])).sum(-1)
    keep = np.isin(lin(allp), lin(points))
    assert keep.sum() == points.shape[0]
    assert np.array_equal(allp[keep], points)
    enc.keep.copy_(torch.from_numpy(keep).long())
    return enc.eval()


def main():
    ref = ref_import.load()
    build_ref.build_clib()
    gs = np.load(os.path.join(HERE, "golden_small.npz"))
    g = {}
    vs = float(gs["voxel_size"])
    march = vs / 8
    hit = gs["svo_hits"][0]
    I = torch.from_numpy(gs["svo_intersected_voxel_idx"][0][hit])
    L = torch.from_numpy(gs["svo_min_depth"][0][hit])
    U = torch.from_numpy(gs["svo_max_depth"][0][hit])
    N = I.shape[0]

    # parallel sampler: deterministic, then seeded with the jitter recorded
    out = ref.clib._parallel_ray_sampling(march, I, L, U, deterministic=True)
    for k, v in zip(["idx", "depth", "dists"], out):
        g["par_det_%s" % k] = v.numpy()
    first = L.min(1)[0]
    last = U.masked_fill(U.eq(10000.0), 0).max(1)[0]
    K = int((last - first).max() / march)
    torch.manual_seed(5)
    g["par_noise"] = torch.zeros(N, K).uniform_().clamp(min=0.01, max=0.99).numpy()
    torch.manual_seed(5)
    out = ref.clib._parallel_ray_sampling(march, I, L, U, deterministic=False)
    for k, v in zip(["idx", "depth", "dists"], out):
        g["par_rand_%s" % k] = v.numpy()
    g["par_march"] = np.float32(march)

    # uniform op wrapper
    max_len = 4.0
    out = ref.clib.uniform_ray_sampling(I, L, U, march, max_len, True)
    for k, v in zip(["idx", "depth", "dists"], out):
        g["uni_det_%s" % k] = v.numpy()
    Hp = int(np.ceil(N / 256)) * 256
    steps = int(max_len / march) + 2 * I.shape[1]
    torch.manual_seed(6)
    g["uni_noise"] = torch.zeros(256, Hp // 256, steps).uniform_().reshape(Hp, steps).numpy()
    torch.manual_seed(6)
    out = ref.clib.uniform_ray_sampling(I, L, U, march, max_len, False)
    for k, v in zip(["idx", "depth", "dists"], out):
        g["uni_rand_%s" % k] = v.numpy()
    g["uni_max_len"] = np.float32(max_len)

    # ball intersection
    pts = torch.from_numpy(gs["points"])[None]
    rs = torch.from_numpy(gs["ray_start"]).reshape(1, 1, 3).expand(1, gs["ray_dir"].shape[0], 3)
    rd = torch.from_numpy(gs["ray_dir"])[None]
    out = ref.clib.ball_ray_intersect(0.15, 20, pts, rs.contiguous(), rd.contiguous())
    for k, v in zip(["idx", "min", "max"], out):
        g["ball_%s" % k] = v.numpy()
    g["ball_radius"] = np.float32(0.15)

    # c2 subset
    p, vs2 = scenes.scene_shell(1.0 / 64)
    enc = c2_encoder(ref, p, vs2)
    st = enc.precompute(id=None)
    rs2, rd2 = scenes.frame_view(0, size=800)
    ij = np.stack(np.meshgrid(np.arange(200, 600), np.arange(200, 600), indexing="ij"), -1).reshape(-1, 2)
    sel = np.sort(np.random.RandomState(11).choice(ij.shape[0], 6000, replace=False))
    pix = ij[sel, 0] * 800 + ij[sel, 1]
    g["c2_pixels"] = pix.astype(np.int64)
    g["c2_ray_start"] = rs2
    g["c2_ray_dir"] = rd2[pix]
    R = pix.size
    o3 = torch.from_numpy(rs2).reshape(1, 1, 3).expand(1, R, 3).contiguous()
    d3 = torch.from_numpy(rd2[pix]).reshape(1, R, 3).contiguous()
    cen = st["voxel_octree_center_xyz"]
    chi = st["voxel_octree_children_idx"]
    g["c2_octree_centers"] = cen.numpy()
    g["c2_octree_children"] = chi.numpy()
    raw = ref_import.CpuExt.svo_intersect(o3, d3, cen[None].float(), chi[None].int(), vs2, 64)
    for k, v in zip(["idx", "min", "max"], raw):
        g["c2_raw_%s" % k] = v.numpy()
    _, _, out, hits = enc.ray_intersect(torch.from_numpy(rs2).reshape(1, 1, 1, 3),
                                        d3.reshape(1, 1, R, 3),
                                        {k: (v.unsqueeze(0) if v is not None else None)
                                         for k, v in st.items()})
    for k in ["intersected_voxel_idx", "min_depth", "max_depth"]:
        g["c2_%s" % k] = out[k].numpy()
    g["c2_hits"] = hits.numpy()
    d = (out["max_depth"] - out["min_depth"]).masked_fill(out["intersected_voxel_idx"].eq(-1), 0)
    out["probs"] = d / d.sum(dim=-1, keepdim=True)
    out["steps"] = d.sum(-1) / enc.step_size
    g["c2_probs"] = out["probs"].numpy()
    g["c2_steps"] = out["steps"].numpy()
    h = hits.reshape(-1)
    sub = {k: v.reshape(-1, v.shape[-1])[h] if v.dim() == 3 else v.reshape(-1)[h]
           for k, v in out.items()}
    smp = enc.ray_sample(sub)
    for k, v in smp.items():
        g["c2_det_%s" % k] = v.numpy()
    out = ref.clib.parallel_ray_sampling(float(enc.step_size), sub["intersected_voxel_idx"],
                                         sub["min_depth"], sub["max_depth"], True)
    for k, v in zip(["idx", "depth", "dists"], out):
        g["c2_par_%s" % k] = v.numpy()
    np.savez_compressed(os.path.join(HERE, "golden_ops.npz"), **g)
    print("wrote golden_ops.npz: %d c1 hit rays, %d c2 rays (%d hit)" % (N, R, int(h.sum())))


if __name__ == "__main__":
    main()
