"""The leaf-grid SVO intersection (nsvf_svo_intersect_grid) gives the sorted
hit lists of the depth-first traversal + the encoder's stable depth sort
(fairnr/clib/src/intersect_gpu.cu:170-237, fairnr/modules/encoder.py:
518-524), bit for bit:

* the whole c2 frame (800x800) against the oracle's traversal + sort;
* against the depth-first kernel on rays from outside and inside the grid,
  rays along grid planes and axis-aligned rays (a zero direction component:
  listed for the depth-first kernel), a small n_max (rows that overflow:
  listed), voxel sizes whose FP32 faces do not nest (flagged leaves: explicit
  ancestor tests), and the c4 scene;
* the served frame through either traversal."""
import numpy as np
import pytest
import torch

from oracle import cpu, workload

pytestmark = pytest.mark.gpu


def _np(t):
    return t.detach().cpu().numpy()


def _bits(a):
    a = np.asarray(a)
    return a.view(np.int32) if a.dtype == np.float32 else a


def _grid(sc, cuda):
    from nsvf_gb300 import ext
    cen, chi = sc["octree"]
    g = ext.SvoGrid(torch.from_numpy(cen).to(cuda), torch.from_numpy(chi).to(cuda),
                    sc["voxel_size"])
    assert g.ok
    return g


def _check_vs_dfs(g, sc, o, d, n_max, cuda):
    """Grid vs the depth-first kernel on the same rays; returns the hit count."""
    from nsvf_gb300 import ext
    cen, chi = sc["octree"]
    ro = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(o, d.shape), np.float32)).to(cuda)
    rd = torch.from_numpy(np.ascontiguousarray(d, np.float32)).to(cuda)
    got = ext.svo_intersect_grid(g, ro, rd, n_max)
    ref = ext.svo_intersect_sorted(ro[None], rd[None], torch.from_numpy(cen)[None].to(cuda),
                                   torch.from_numpy(chi)[None].to(cuda), sc["voxel_size"], n_max)
    for a, b, what in zip(got, ref, ["idx", "min_depth", "max_depth", "hits"]):
        assert np.array_equal(_bits(_np(a)), _bits(_np(b))), what
    ext.check_errors(cuda)
    return int((_np(got[0]) != -1).sum())


@pytest.fixture(scope="module")
def c2():
    return workload.c2_scene(1.0 / 64)


def test_c2_frame_matches_oracle(c2, cuda):
    from nsvf_gb300 import ext
    g = _grid(c2, cuda)
    cen, chi = c2["octree"]
    o, d = workload.frame(0)
    ro = np.ascontiguousarray(np.broadcast_to(o, d.shape), np.float32)
    got = ext.svo_intersect_grid(g, torch.from_numpy(ro).to(cuda), torch.from_numpy(d).to(cuda), 64)
    ref = cpu.sort_hits(*cpu.svo_intersect(ro[None], d[None], cen[None], chi[None],
                                           c2["voxel_size"], 64))
    for a, b, what in zip(got[:3], ref, ["idx", "min_depth", "max_depth"]):
        assert np.array_equal(_bits(_np(a)), _bits(b)), what
    assert np.array_equal(_np(got[3])[0], (ref[0][0] != -1).any(-1))
    assert int(_np(got[3]).sum()) > 100000
    ext.check_errors(cuda)


def _inside_rays(n, seed):
    rng = np.random.RandomState(seed)
    o = rng.uniform(-1, 1, (n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def _plane_rays(n, seed, vs):
    """Origins on grid planes, directions along an axis (some exactly: zero
    components) or nearly."""
    rng = np.random.RandomState(seed)
    d = np.zeros((n, 3), np.float64)
    d[np.arange(n), rng.randint(0, 3, n)] = rng.choice([-1.0, 1.0], n)
    d += (rng.rand(n, 3) < 0.5) * 1e-3 * rng.randint(0, 2, (n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.round(rng.uniform(-1.2, 1.2, (n, 3)) / (vs / 2)) * (vs / 2)
    return o.astype(np.float32), d.astype(np.float32)


@pytest.mark.parametrize("n_max", [64, 8])
def test_unpadded_rows_gather_the_same(c2, cuda, n_max):
    """nsvf_svo_intersect_grid_rows without padding (the served chain's form)
    on the c2 frame: hit flags equal; a hit ray's row holds the padded call's
    hits and then a -1; a missed ray's row is not written; and
    nsvf_gather_probs turns both forms into the same bits (n_max 8: rows of
    overflow and listed rays, which are complete either way)."""
    from nsvf_gb300 import ext
    from nsvf_gb300._lib import LIB
    g = _grid(c2, cuda)
    o, d = workload.frame(0)
    R = d.shape[0]
    ro = torch.from_numpy(np.ascontiguousarray(np.broadcast_to(o, d.shape), np.float32)).to(cuda)
    rd = torch.from_numpy(d).to(cuda)
    ref = ext.svo_intersect_grid(g, ro, rd, n_max)
    idx = torch.full((R, n_max), 7777, dtype=torch.int32, device=cuda)
    lo = torch.full((R, n_max), float("nan"), device=cuda)
    hi = torch.full((R, n_max), float("nan"), device=cuda)
    hits = torch.full((R,), 9, dtype=torch.uint8, device=cuda)
    stream = ext.ctypes_stream(cuda)
    g.intersect_into(R, n_max, ro.data_ptr(), rd.data_ptr(), idx.data_ptr(), lo.data_ptr(),
                     hi.data_ptr(), hits.data_ptr(), stream, padded=False)
    ext.check_errors(cuda)
    r_idx = ref[0].reshape(R, n_max)
    assert torch.equal(hits, ref[3].reshape(R).to(torch.uint8))
    cnt = (r_idx != -1).sum(1)
    hit = hits.bool()
    assert int(hit.sum()) > 100000
    valid = torch.arange(n_max, device=cuda)[None, :] < cnt[:, None]
    assert torch.equal(idx[valid], r_idx[valid])
    assert torch.equal(lo[valid], ref[1].reshape(R, n_max)[valid])
    assert torch.equal(hi[valid], ref[2].reshape(R, n_max)[valid])
    term = hit & (cnt < n_max)
    assert bool((idx[term, :].gather(1, cnt[term, None]) == -1).all())
    assert bool((idx[~hit] == 7777).all())
    pix = torch.nonzero(hit).reshape(-1)
    n_hit = torch.tensor([pix.numel()], dtype=torch.int64, device=cuda)

    def gathered(i_, l_, h_):
        n = pix.numel()
        out = [torch.empty(n, n_max, dtype=torch.int32, device=cuda)] + \
            [torch.empty(n, n_max, device=cuda) for _ in range(3)] + [torch.empty(n, device=cuda)]
        assert LIB.nsvf_gather_probs(n, n_hit.data_ptr(), n_max, 1.0 / 512, pix.data_ptr(),
                                     i_.data_ptr(), l_.data_ptr(), h_.data_ptr(),
                                     *[t.data_ptr() for t in out], stream) == 0
        return out

    a = gathered(*(t.reshape(R, n_max).contiguous() for t in ref[:3]))
    b = gathered(idx, lo, hi)
    for x, y in zip(a, b):
        assert np.array_equal(_bits(_np(x)), _bits(_np(y)))


@pytest.mark.parametrize("case", ["camera", "inside", "planes", "small_n_max"])
def test_c2_matches_dfs_kernel(c2, cuda, case):
    g = _grid(c2, cuda)
    if case == "camera":
        o, d = workload.frame(37)
        sel = np.random.RandomState(1).choice(d.shape[0], 200000, replace=False)
        assert _check_vs_dfs(g, c2, o, d[sel], 64, cuda) > 500000
    elif case == "inside":
        o, d = _inside_rays(60000, 2)
        assert _check_vs_dfs(g, c2, o, d, 64, cuda) > 100000
    elif case == "planes":
        o, d = _plane_rays(60000, 3, c2["voxel_size"])
        assert _check_vs_dfs(g, c2, o, d, 64, cuda) > 10000
    else:
        o, d = workload.frame(5)
        sel = np.random.RandomState(2).choice(d.shape[0], 100000, replace=False)
        assert _check_vs_dfs(g, c2, o, d[sel], 8, cuda) > 100000


@pytest.mark.parametrize("vs", [1.0 / 50, 0.037])
def test_flagged_leaves_match_dfs_kernel(cuda, vs):
    sc = {"voxel_size": vs, "octree": workload.octree(workload.shell_points(vs), vs / 2)}
    g = _grid(sc, cuda)
    assert g.n_flagged > 0
    o, d = workload.frame(3)
    sel = np.random.RandomState(4).choice(d.shape[0], 100000, replace=False)
    _check_vs_dfs(g, sc, o, d[sel], 64, cuda)
    o, d = _inside_rays(30000, 5)
    _check_vs_dfs(g, sc, o, d, 64, cuda)


def test_c4_matches_dfs_kernel(cuda):
    sc = {"voxel_size": 1.0 / 128,
          "octree": workload.octree(workload.shell_points(1.0 / 128), 1.0 / 256)}
    g = _grid(sc, cuda)
    o, d = workload.frame(0)
    sel = np.random.RandomState(6).choice(d.shape[0], 200000, replace=False)
    assert _check_vs_dfs(g, sc, o, d[sel], 64, cuda) > 500000


def test_served_frame_same_with_either_traversal(cuda):
    import argparse
    from nsvf_gb300 import scenes, served
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    p, vs = scenes.scene_shell(1.0 / 64)
    args = argparse.Namespace(voxel_size=vs, max_hits=64, raymarching_stepsize_ratio=0.125,
                              voxel_embed_dim=32, use_octree=True, deterministic_step=True)
    enc = SparseVoxelEncoder(args, points=p)
    with torch.no_grad():
        enc.values.weight.copy_(scenes.voxel_embeddings(enc.values.weight.shape[0], 32, 0.01,
                                                        seed=1))
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=2))
    scene = served.SceneState(enc.to(cuda).eval(), field.to(cuda).eval())
    assert scene.svo_grid.ok
    ro, rd = scenes.frame_view(2, size=400)
    ro = torch.from_numpy(ro).to(cuda)
    rd = torch.from_numpy(rd).to(cuda)
    a = served.render_frame(scene, ro, rd, traversal="grid")
    a = {k: (v.clone() if torch.is_tensor(v) else v) for k, v in a.items()}
    b = served.render_frame(scene, ro, rd, traversal="dfs")
    for k in ["colors", "depths", "missed"]:
        assert torch.equal(a[k], b[k]), k
    assert a["n_samples"] == b["n_samples"] > 0
