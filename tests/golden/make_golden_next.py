"""Golden fixtures for the steps either side of the rendering path, from the
reference itself (run where the reference checkout is present):

    python tests/golden/make_golden_next.py

Writes golden_next.npz, on the 147-voxel "small" scene of golden_small.npz:

* rays_* -- ray generation: get_uv (fairnr/data/data_utils.py:57-65) on a
  64x64 image read at 32x32, and get_ray_direction
  (fairnr/data/geometry.py:116-122) for a seeded camera (intrinsics,
  camera-to-world matrix);
* es_* -- VolumeRenderer with raymarching_tolerance 0.01 and 1,024-sample
  column chunks: the early-terminating column loop
  (fairnr/modules/renderer.py:146-188) on the deterministic samples;
* split_* -- SparseVoxelEncoder.splitting (fairnr/modules/encoder.py:656-676):
  new voxel centres, corner ids and re-interpolated corner embeddings.
* rf_* -- a seeded reference RaidanceField (inputs "emb:6:32" / "feat:0:64,
  ray:4", widths 64/32/64, 1 feature layer, 2 texture layers) rendering the
  deterministic samples with the reference's VolumeRenderer: its state dict
  (rf_state_<name>) and colors/depths/missed;
* tri_* -- triangle_ray_intersect (fairnr/clib/__init__.py:136-173) of the
  c1 camera's rays against a seeded closed mesh (an icosphere-like cage of
  320 faces, radius 0.7) with cagesize 0.05, blur 0.01, n_max 8.
"""
import argparse
import os
import sys

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from oracle import ref_import, build_ref  # noqa: E402
from nsvf_gb300 import scenes  # noqa: E402
import make_golden as mg  # noqa: E402


def cage_mesh(radius=0.7, subdiv=2, seed=3):
    """A closed triangle cage: an icosahedron subdivided twice (320 faces),
    vertices on a sphere of `radius` with a seeded 5 % radial jitter."""
    t = (1.0 + 5 ** 0.5) / 2.0
    v = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t),
         (0, 1, -t), (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    f = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9),
         (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    verts = [np.array(x, np.float64) / np.linalg.norm(x) for x in v]
    for _ in range(subdiv):
        mid = {}
        nf = []
        for a, b, c in f:
            ids = []
            for p, q in ((a, b), (b, c), (c, a)):
                key = (min(p, q), max(p, q))
                if key not in mid:
                    m = verts[p] + verts[q]
                    verts.append(m / np.linalg.norm(m))
                    mid[key] = len(verts) - 1
                ids.append(mid[key])
            nf += [(a, ids[0], ids[2]), (b, ids[1], ids[0]), (c, ids[2], ids[1]), tuple(ids)]
        f = nf
    rng = np.random.RandomState(seed)
    V = np.array(verts) * radius * (1 + 0.05 * rng.uniform(-1, 1, size=(len(verts), 1)))
    return V.astype(np.float32), np.array(f, np.int64)


def main():
    ref = ref_import.load()
    build_ref.build_clib()
    du = sys.modules["fairnr.data.data_utils"]
    torch.manual_seed(0)
    g = {}
    # --- ray generation -------------------------------------------------
    cam = scenes.sphere_cameras(1, 4.0, 5)[0]
    R = scenes.look_at(np.asarray(cam, np.float64))
    inv_RT = np.eye(4, dtype=np.float32)
    inv_RT[:3, :3] = R
    inv_RT[:3, 3] = cam
    intr = np.array([80.0, 78.0, 31.5, 32.5], np.float32)      # fx, fy, cx, cy
    uv, ratio = du.get_uv(64, 64, 32, 32)                       # read 64x64 at 32x32
    uv_t = torch.from_numpy(np.ascontiguousarray(uv)).reshape(2, -1)
    K = np.eye(4, dtype=np.float32)
    K[0, 0], K[1, 1], K[0, 2], K[1, 2] = intr
    inv_RT_t = torch.from_numpy(inv_RT)
    ray_start = inv_RT_t[:3, 3]
    ray_dir = ref.geometry.get_ray_direction(ray_start, uv_t, torch.from_numpy(K), inv_RT_t)
    g["rays_intrinsics"] = intr
    g["rays_inv_RT"] = inv_RT
    g["rays_uv"] = uv_t.numpy()
    g["rays_hw"] = np.array([64, 64, 32, 32], np.int64)          # H, W, h, w
    g["rays_start"] = ray_start.numpy()
    g["rays_dir"] = ray_dir.t().contiguous().numpy()
    # --- early-terminating renderer --------------------------------------
    pts, vs = scenes.scene_small()
    rs, rd = scenes.small_view(0)
    embed = scenes.voxel_embeddings(1000, 32, std=1.0, seed=1)
    weights = scenes.stand_in_mlp_weights(seed=2, sigma_scale=mg.GOLDEN_SIGMA_SCALE,
                                          sigma_bias=mg.GOLDEN_SIGMA_BIAS)
    field = mg.StandInField(weights).eval()
    enc = mg.make_encoder(ref, pts, vs, True, embed)
    st = enc.precompute(id=None)
    sel = np.arange(0, rd.shape[0], 4)
    ray_dir = torch.from_numpy(rd[sel]).reshape(1, 1, -1, 3)
    ray_start = torch.from_numpy(rs).reshape(1, 1, 1, 3)
    _, _, out, hits = enc.ray_intersect(ray_start, ray_dir, {
        k: (v.unsqueeze(0) if v is not None else None) for k, v in st.items()})
    out = mg.probs_steps(out, enc.step_size)
    h = hits.reshape(-1)
    sub = {k: v.reshape(-1, v.shape[-1])[h] if v.dim() == 3 else v.reshape(-1)[h]
           for k, v in out.items()}
    samples = enc.ray_sample(sub)
    N = int(h.sum())
    rsh = ray_start.reshape(1, 3).expand(N, 3)
    rdh = ray_dir.reshape(-1, 3)[h]
    for tol in (0.01, 0.5):
        ren = ref.renderer.VolumeRenderer(argparse.Namespace(chunk_size=1, raymarching_tolerance=tol)).eval()
        with torch.no_grad():
            res = ren(enc, field, rsh, rdh, dict(samples), st)
        tag = "es%g" % tol
        for k in ["colors", "depths", "missed", "probs"]:
            g["%s_%s" % (tag, k)] = res[k].detach().numpy()
        g["%s_ae" % tag] = np.int64(int(res["ae"]))
    # --- a reference radiance field rendering the same samples -----------
    torch.manual_seed(11)
    rf_args = argparse.Namespace(inputs_to_density="emb:6:32", inputs_to_texture="feat:0:64, ray:4",
                                 feature_embed_dim=64, density_embed_dim=32, texture_embed_dim=64,
                                 feature_layers=1, texture_layers=2, background_stop_gradient=False)
    rf = ref.field.RaidanceField(rf_args).eval()
    with torch.no_grad():
        rf.predictor.output_layer.bias.fill_(0.5)          # a partly opaque scene
    ren = ref.renderer.VolumeRenderer(argparse.Namespace(chunk_size=64)).eval()
    with torch.no_grad():
        res = ren(enc, rf, rsh, rdh, dict(samples), st)
    for k, v in rf.state_dict().items():
        g["rf_state_" + k] = v.numpy()
    for k in ["colors", "depths", "missed"]:
        g["rf_%s" % k] = res[k].detach().numpy()
    # --- splitting --------------------------------------------------------
    enc_s = mg.make_encoder(ref, pts, vs, True, embed)
    enc_s.splitting()
    g["split_points"] = enc_s.points.numpy()
    g["split_feats"] = enc_s.feats.numpy()
    g["split_values"] = enc_s.values.weight.detach().numpy()
    g["split_num_keys"] = np.int64(int(enc_s.num_keys))
    g["split_keep"] = enc_s.keep.numpy()
    # --- triangle intersection (mesh encoder op) ---------------------------
    verts, faces = cage_mesh()
    rs_t = torch.from_numpy(np.broadcast_to(rs, rd[sel].shape).copy()).reshape(1, -1, 3)
    rd_t = torch.from_numpy(rd[sel]).reshape(1, -1, 3)
    inds, depth, uv = ref.clib.triangle_ray_intersect(0.05, 0.01, 8, torch.from_numpy(verts),
                                                      torch.from_numpy(faces), rs_t, rd_t)
    g["tri_verts"] = verts
    g["tri_faces"] = faces
    g["tri_ray_start"] = rs_t.numpy()
    g["tri_ray_dir"] = rd_t.numpy()
    g["tri_inds"] = inds.numpy()
    g["tri_depth"] = depth.numpy()
    g["tri_uv"] = uv.numpy()
    np.savez_compressed(os.path.join(HERE, "golden_next.npz"), **g)
    print("wrote golden_next.npz", {k: getattr(v, "shape", None) for k, v in g.items()})
    print("early stop evals:", int(g["es0.01_ae"]), int(g["es0.5_ae"]))


if __name__ == "__main__":
    main()
