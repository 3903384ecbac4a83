"""Parity of the sm_103a ops (through the C ABI, via nsvf_gb300.ext / clib)
with the CPU oracle and the golden fixtures made from the reference.

Integer outputs (voxel ids, sample-to-voxel assignments) and the FP32 depths
of intersection and sampling are compared bit for bit: both sides run the
reference's FP32 operation sequence (see include/nsvf_gb300.h)."""
import numpy as np
import pytest
import torch

from oracle import cpu

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _np(t):
    return t.detach().cpu().numpy()


def _rays_golden(g, dev):
    R = g["ray_dir"].shape[0]
    rs = np.broadcast_to(g["ray_start"], (R, 3))[None].astype(np.float32)
    return _t(rs, dev), _t(g["ray_dir"][None], dev)


def test_aabb_matches_golden(golden, cuda):
    from nsvf_gb300 import ext
    g = golden
    rs, rd = _rays_golden(g, cuda)
    out = ext.aabb_intersect(rs, rd, _t(g["aabb_centers_shifted"][None], cuda),
                             float(g["voxel_size"]), 20)
    for got, key in zip(out, ["aabb_raw_idx", "aabb_raw_min", "aabb_raw_max"]):
        assert np.array_equal(_np(got), g[key]), key


def test_svo_matches_golden(golden, cuda):
    from nsvf_gb300 import ext
    g = golden
    rs, rd = _rays_golden(g, cuda)
    pts, chi = _t(g["octree_centers"][None], cuda), _t(g["octree_children"][None], cuda)
    out = ext.svo_intersect(rs, rd, pts, chi, float(g["voxel_size"]), 20)
    for got, key in zip(out, ["svo_raw_idx", "svo_raw_min", "svo_raw_max"]):
        assert np.array_equal(_np(got), g[key]), key
    idx, lo, hi, hits = ext.svo_intersect_sorted(rs, rd, pts, chi, float(g["voxel_size"]), 20)
    oi, ol, oh = cpu.sort_hits(*[g[k] for k in ["svo_raw_idx", "svo_raw_min", "svo_raw_max"]])
    assert np.array_equal(_np(idx), oi) and np.array_equal(_np(lo), ol)
    assert np.array_equal(_np(hi), oh)
    assert np.array_equal(_np(lo), g["svo_min_depth"])
    assert np.array_equal(_np(hits), g["svo_hits"])
    ext.check_errors(cuda)


def _random_rays(n, seed, origin_radius=3.0):
    rng = np.random.RandomState(seed)
    o = rng.normal(size=(n, 3))
    o = o / np.linalg.norm(o, axis=1, keepdims=True) * origin_radius * rng.uniform(0.2, 1.0, (n, 1))
    d = -o + rng.normal(scale=0.4, size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    # a few axis-aligned and degenerate directions (zero components -> inf reciprocals)
    d[:8] = [[1, 0, 0], [0, 1, 0], [0, 0, 1], [-1, 0, 0], [0, -1, 0], [0, 0, -1],
             [0.6, 0.8, 0], [0, 0.6, -0.8]]
    o[:8] = [[-2, 0.1, 0.05], [0.12, -2, 0.0], [0.0, 0.0, -2], [2, 0.25, 0.25],
             [0.5, 2, 0.5], [0.125, 0.125, 2], [-1.5, -1.5, 0.3], [0.2, -0.9, 1.5]]
    return o.astype(np.float32), d.astype(np.float32)


@pytest.mark.parametrize("voxel,n_max", [(1.0 / 16, 4), (1.0 / 16, 64), (1.0 / 32, 64)])
def test_svo_matches_oracle_random_rays(cuda, voxel, n_max):
    from nsvf_gb300 import ext, geometry, scenes
    p, vs = scenes.scene_shell(voxel)
    cen, chi = geometry.build_easy_octree(torch.from_numpy(p), vs / 2)
    o, d = _random_rays(3000, seed=int(1 / voxel) + n_max)
    out = ext.svo_intersect(_t(o[None], cuda), _t(d[None], cuda), cen[None].to(cuda),
                            chi[None].to(cuda), vs, n_max)
    ref = cpu.svo_intersect(o[None], d[None], cen.numpy()[None], chi.numpy()[None], vs, n_max)
    for a, b in zip(out, ref):
        assert np.array_equal(_np(a), b)
    assert (ref[0] != -1).sum() > 1000
    srt = ext.svo_intersect_sorted(_t(o[None], cuda), _t(d[None], cuda), cen[None].to(cuda),
                                   chi[None].to(cuda), vs, n_max)
    rs = cpu.sort_hits(*ref)
    for a, b in zip(srt[:3], rs):
        assert np.array_equal(_np(a), b)
    if n_max == 64:
        # both sort paths: rows of at most 32 hits sort as 32 slots, longer
        # rows through the whole 64-slot network
        cnt = (ref[0][0] != -1).sum(-1)
        assert (cnt > 32).sum() > 100 and ((cnt > 0) & (cnt <= 32)).sum() > 1000
    ext.check_errors(cuda)


def _mixed_tree(seed, depth=5, hv=0.02):
    """A random octree whose nodes mix leaf and internal children at every
    depth (build_octree never makes one: its leaves all hang under depth-0
    nodes). Post-order numbering puts the root last, as the reference's
    flattening does; children[8] is the node size (1 = leaf)."""
    rng = np.random.RandomState(seed)
    cen, chi = [], []

    def make(c, lvl, d):
        if lvl == 0:
            cen.append(c)
            chi.append([-1] * 8 + [1])
            return len(cen) - 1
        kids = []
        for j in range(8):
            s = np.array([(j >> 2) & 1, (j >> 1) & 1, j & 1]) * 2 - 1
            cc = c + s * hv * (2 ** lvl) / 2
            r = rng.rand()
            if r < 0.3:
                kids.append(-1)
            elif r < 0.55 or d == depth:
                kids.append(make(cc, 0, d + 1))
            else:
                kids.append(make(cc, lvl - 1, d + 1))
        cen.append(c)
        chi.append(kids + [2 ** lvl])
        return len(cen) - 1

    make(np.zeros(3), depth, 0)
    return np.array(cen, np.float32), np.array(chi, np.int32)


@pytest.mark.parametrize("seed,n_max", [(5, 32), (6, 8), (7, 128)])
def test_svo_mixed_children_matches_oracle(cuda, seed, n_max):
    """Nodes with both leaf and internal hit children: leaves met on the
    descent stack are emitted one at a time, in the reference's DFS order."""
    from nsvf_gb300 import ext
    cen, chi = _mixed_tree(seed)
    vs = 0.04
    rng = np.random.RandomState(seed + 100)
    o = rng.normal(size=(2000, 3))
    o = (3 * o / np.linalg.norm(o, axis=1, keepdims=True)).astype(np.float32)
    d = -o + rng.normal(scale=0.2, size=(2000, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    args = (_t(o[None], cuda), _t(d[None], cuda), _t(cen[None], cuda), _t(chi[None], cuda), vs, n_max)
    ref = cpu.svo_intersect(o[None], d[None], cen[None], chi[None], vs, n_max)
    for a, b in zip(ext.svo_intersect(*args), ref):
        assert np.array_equal(_np(a), b)
    assert (ref[0] != -1).sum() > 1000
    for a, b in zip(ext.svo_intersect_sorted(*args)[:3], cpu.sort_hits(*ref)):
        assert np.array_equal(_np(a), b)
    ext.check_errors(cuda)


def test_aabb_matches_oracle_many_voxels(cuda):
    """More voxels than one shared-memory tile, rays in two batch rows with
    their own voxel copies."""
    from nsvf_gb300 import ext, scenes
    p, vs = scenes.scene_shell(1.0 / 16)
    assert p.shape[0] > 1024
    o, d = _random_rays(600, seed=7)
    o2, d2 = o.reshape(2, 300, 3), d.reshape(2, 300, 3)
    pts = np.stack([p, p[::-1].copy()])
    out = ext.aabb_intersect(_t(o2, cuda), _t(d2, cuda), _t(pts, cuda), vs, 12)
    ref = cpu.aabb_intersect(o2, d2, pts, vs, 12)
    for a, b in zip(out, ref):
        assert np.array_equal(_np(a), b)
    # shared voxel set (b_pts = 1) equals the copied one
    out1 = ext.aabb_intersect(_t(o2, cuda), _t(d2, cuda), _t(p[None], cuda), vs, 12)
    ref1 = cpu.aabb_intersect(o2, d2, np.stack([p, p]), vs, 12)
    for a, b in zip(out1, ref1):
        assert np.array_equal(_np(a), b)


def test_ball_matches_oracle(cuda):
    from nsvf_gb300 import ext, scenes
    p, vs = scenes.scene_small()
    o, d = _random_rays(500, seed=3)
    out = ext.ball_intersect(_t(o[None], cuda), _t(d[None], cuda), _t(p[None], cuda), 0.2, 10)
    ref = cpu.ball_intersect(o[None], d[None], p[None], 0.2, 10)
    assert np.array_equal(_np(out[0]), ref[0])
    np.testing.assert_array_equal(_np(out[1]), ref[1])
    np.testing.assert_array_equal(_np(out[2]), ref[2])


def _hit_rows(g):
    hit = g["svo_hits"][0]
    return [g[k][0][hit] for k in ["svo_intersected_voxel_idx", "svo_min_depth",
                                   "svo_max_depth", "svo_probs"]] + [g["svo_steps"][0][hit]]


def _post(si, sd, ss):
    ss = ss.clamp(min=0.0)
    sd = sd.masked_fill(si.eq(-1), 10000.0)
    ss = ss.masked_fill(si.eq(-1), 0.0)
    return si, sd, ss


def test_inverse_cdf_matches_golden(golden, cuda):
    from nsvf_gb300 import clib, ext
    g = golden
    I, lo, hi, pr, st = [_t(a, cuda) for a in _hit_rows(g)]
    si, sd, ss = _post(*clib.inverse_cdf_sampling(I, lo, hi, pr, st, -1, True))
    assert np.array_equal(_np(si), g["svo_det_sampled_point_voxel_idx"])
    assert np.array_equal(_np(sd), g["svo_det_sampled_point_depth"])
    assert np.array_equal(_np(ss), g["svo_det_sampled_point_distance"])
    # recorded seeded noise, the wrapper's launch layout
    N = I.shape[0]
    noise = _t(g["svo_noise"], cuda)
    si, sd, ss = ext.inverse_cdf_sampling_rows(I, lo, hi, noise, pr, st, -1.0,
                                               clib.inverse_cdf_layout(N), noise.shape[1])
    L = int(si.ne(-1).sum(-1).max())
    si, sd, ss = _post(si[:, :L], sd[:, :L], ss[:, :L])
    assert np.array_equal(_np(si), g["svo_rand_sampled_point_voxel_idx"])
    assert np.array_equal(_np(sd), g["svo_rand_sampled_point_depth"])
    assert np.array_equal(_np(ss), g["svo_rand_sampled_point_distance"])


def _random_intervals(rows, H, seed, full_rows=0.2):
    """Sorted, padded hit lists like the encoder produces; `full_rows` of the
    rows use all H slots (the tail-read case)."""
    rng = np.random.RandomState(seed)
    idx = np.full((rows, H), -1, np.int32)
    lo = np.full((rows, H), 10000.0, np.float32)
    hi = np.full((rows, H), 10000.0, np.float32)
    for r in range(rows):
        n = H if rng.rand() < full_rows else rng.randint(1, H + 1)
        starts = np.sort(rng.uniform(1.0, 6.0, n)).astype(np.float32)
        lens = rng.uniform(0.01, 0.3, n).astype(np.float32)
        idx[r, :n] = rng.randint(0, 5000, n)
        lo[r, :n] = starts
        hi[r, :n] = starts + lens
    d = np.where(idx == -1, 0, hi - lo).astype(np.float32)
    probs = (d / d.sum(-1, keepdims=True)).astype(np.float32)
    steps = (d.sum(-1) / np.float32(0.02)).astype(np.float32)
    return idx, lo, hi, probs, steps


@pytest.mark.parametrize("b,m,H", [(3, 50, 8), (1, 257, 16), (5, 1, 4)])
def test_inverse_cdf_raw_op_matches_oracle(cuda, b, m, H):
    from nsvf_gb300 import ext
    idx, lo, hi, probs, steps = _random_intervals(b * m, H, seed=b * 100 + m)
    M = int(np.ceil(steps).max()) + H
    noise = np.random.RandomState(1).uniform(0.001, 0.999, (b * m, M)).astype(np.float32)
    sh = lambda a: a.reshape(b, m, *a.shape[1:])
    out = ext.inverse_cdf_sampling(*[_t(sh(a), cuda) for a in (idx, lo, hi)],
                                   _t(sh(noise), cuda), _t(sh(probs), cuda), _t(sh(steps), cuda),
                                   -1.0)
    ref = cpu.inverse_cdf_sampling(sh(idx), sh(lo), sh(hi), sh(noise), sh(probs), sh(steps), -1.0)
    for a, r in zip(out, ref):
        assert np.array_equal(_np(a), r)
    ext.check_errors(cuda)


@pytest.mark.parametrize("N", [1, 199, 1001, 2500])
def test_inverse_cdf_wrapper_layout_matches_oracle(cuda, N):
    """Rays blocked as the reference wrapper does (200 blocks, 800-column
    launches): the tail and next-row reads depend on that layout."""
    from nsvf_gb300 import clib, ext
    H = 6
    idx, lo, hi, probs, steps = _random_intervals(N, H, seed=N, full_rows=0.5)
    M = int(np.ceil(steps).max()) + H
    Hp = int(np.ceil(N / 200)) * 200
    noise = np.random.RandomState(2).uniform(0.001, 0.999, (Hp, M)).astype(np.float32)
    out = ext.inverse_cdf_sampling_rows(*[_t(a, cuda) for a in (idx, lo, hi)], _t(noise, cuda),
                                        _t(probs, cuda), _t(steps, cuda), -1.0,
                                        clib.inverse_cdf_layout(N), M)
    ref = cpu.inverse_cdf_op(idx, lo, hi, probs, steps, noise)
    L = ref[0].shape[1]
    for a, r in zip(out, ref):
        assert np.array_equal(_np(a)[:, :L], r)


def test_uniform_sampling_matches_oracle(cuda):
    from nsvf_gb300 import ext
    H = 8
    idx, lo, hi, probs, steps = _random_intervals(300, H, seed=11)
    step = 0.02
    M = int((hi[idx != -1].max() - lo[:, 0].min()) / step) + 2 * H
    noise = np.random.RandomState(4).rand(1, 300, M).astype(np.float32)
    out = ext.uniform_ray_sampling(_t(idx[None], cuda), _t(lo[None], cuda), _t(hi[None], cuda),
                                   _t(noise, cuda), step, M)
    ref = cpu.uniform_ray_sampling(idx[None], lo[None], hi[None], noise, step, M)
    for a, r in zip(out, ref):
        assert np.array_equal(_np(a), r)


def test_edge_cases(cuda):
    from nsvf_gb300 import ext, geometry, scenes
    p, vs = scenes.scene_small()
    cen, chi = geometry.build_easy_octree(torch.from_numpy(p), vs / 2)
    cen, chi = cen[None].to(cuda), chi[None].to(cuda)
    # empty ray batch
    e = torch.zeros(1, 0, 3, device=cuda)
    out = ext.svo_intersect(e, e, cen, chi, vs, 8)
    assert out[0].shape == (1, 0, 8)
    # rays that miss everything (pointing away) and n_max = 1
    o = torch.tensor([[[3.0, 3.0, 3.0], [0.0, 0.0, 5.0]]], device=cuda)
    d = torch.tensor([[[1.0, 0.0, 0.0], [0.0, 0.0, 1.0]]], device=cuda)
    idx, lo, hi = ext.svo_intersect(o, d, cen, chi, vs, 1)
    assert (idx == -1).all() and (lo == 0).all()
    # wrong dtype / layout raise like the reference's TORCH_CHECK
    with pytest.raises(RuntimeError):
        ext.svo_intersect(o.double(), d, cen, chi, vs, 8)
    strided = torch.zeros(1, 2, 6, device=cuda)[..., ::2]
    assert not strided.is_contiguous()
    with pytest.raises(RuntimeError):
        ext.aabb_intersect(strided, d, cen, vs, 8)
    # a malformed octree (child id out of range) is reported, not faulted
    bad = chi.clone()
    bad[0, -1, 0] = 10 ** 6
    ext.svo_intersect(o, -o, cen, bad, vs, 8)
    with pytest.raises(RuntimeError):
        ext.check_errors(cuda)


def test_full_frame_properties(cuda):
    """A full 800x800 frame of the 125k-voxel shell: a random subset of rays
    equals the oracle; sorted output is sorted and consistent with hits."""
    from nsvf_gb300 import ext, geometry, scenes
    p, vs = scenes.scene_shell(1.0 / 64)
    cen, chi = geometry.build_easy_octree(torch.from_numpy(p), vs / 2)
    rs, rd = scenes.frame_view(0)
    R = rd.shape[0]
    o = torch.from_numpy(np.broadcast_to(rs, (R, 3)).copy())[None].to(cuda)
    d = torch.from_numpy(rd)[None].to(cuda)
    idx, lo, hi, hits = ext.svo_intersect_sorted(o, d, cen[None].to(cuda), chi[None].to(cuda),
                                                 vs, 64)
    ext.check_errors(cuda)
    lo_np = _np(lo)[0]
    assert (np.diff(lo_np, axis=-1) >= 0).all()
    assert np.array_equal(_np(hits)[0], (_np(idx)[0] != -1).any(-1))
    assert _np(hits).mean() > 0.1
    sel = np.random.RandomState(0).choice(R, 2000, replace=False)
    ref = cpu.svo_intersect(np.broadcast_to(rs, (2000, 3))[None], rd[sel][None],
                            cen.numpy()[None], chi.numpy()[None], vs, 64)
    ref = cpu.sort_hits(*ref)
    assert np.array_equal(_np(idx)[0][sel], ref[0][0])
    assert np.array_equal(lo_np[sel], ref[1][0])


def _icdf_rows(case, cuda):
    """(pts_idx, min_depth, max_depth) rows for the sampling parity test:
    sorted SVO hit rows of a scene, or synthetic sorted rows (1,000 rows,
    several of the reference wrapper's 200-row blocks; H = 160 exercises the
    per-thread walk used beyond 128 slots)."""
    from nsvf_gb300 import ext, geometry, scenes
    if case == "scene":
        p, vs = scenes.scene_shell(1.0 / 32)
        cen, chi = geometry.build_easy_octree(torch.from_numpy(p), vs / 2)
        o, d = _random_rays(6000, seed=21)
        idx, lo, hi, hits = ext.svo_intersect_sorted(_t(o[None], cuda), _t(d[None], cuda),
                                                     cen[None].to(cuda), chi[None].to(cuda), vs, 64)
        h = hits[0].bool()
        return idx[0][h].contiguous(), lo[0][h].contiguous(), hi[0][h].contiguous(), vs / 8, \
            _t(o, cuda)[h].contiguous(), _t(d, cuda)[h].contiguous()
    H = 20 if case == "synthetic" else 160
    rng = np.random.RandomState(7 if case == "synthetic" else 8)
    n = 1000
    I = np.full((n, H), -1, np.int32)
    lo = np.full((n, H), 10000.0, np.float32)
    hi = np.full((n, H), 10000.0, np.float32)
    for r in range(n):
        k = rng.randint(1, H + 1)
        t = np.sort(rng.uniform(0.5, 4.0, size=2 * k)).astype(np.float32)
        I[r, :k] = rng.randint(0, 5000, size=k)
        lo[r, :k], hi[r, :k] = t[0::2], t[1::2]
        if rng.rand() < 0.1:
            hi[r, :k] = lo[r, :k]                 # rays of zero length inside voxels
    o = rng.normal(size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3)).astype(np.float32)
    return _t(I, cuda), _t(lo, cuda), _t(hi, cuda), 0.02, _t(o, cuda), _t(d, cuda)


@pytest.mark.parametrize("case", ["scene", "synthetic", "synthetic_h160"])
def test_sample_compact_matches_inverse_cdf_op(cuda, case):
    """The served path's sample pass (nsvf_sample_count + nsvf_sample_compact,
    warp per ray; per-thread walk beyond 128 slots) gives exactly the valid
    samples of the reference op's padded rows (deterministic jitter, the
    wrapper's 200-block layout), in row order: ids, depths, clamped
    distances and positions o + d t, bit for bit."""
    import ctypes
    from nsvf_gb300 import clib, ext
    from nsvf_gb300._lib import LIB, check
    I, L, Hh, step, ro, rd = _icdf_rows(case, cuda)
    n, H = I.shape
    d = (Hh - L).masked_fill(I.eq(-1), 0)
    tot = d.sum(-1, keepdim=True)
    keep = tot[:, 0] > 0
    I, L, Hh, ro, rd, d, tot = I[keep], L[keep], Hh[keep], ro[keep], rd[keep], d[keep], tot[keep]
    n = I.shape[0]
    probs = (d / tot).contiguous()
    steps = (tot[:, 0] / step).contiguous()
    si, sd, ss = clib.inverse_cdf_sampling(I, L, Hh, probs, steps, -1, True)
    valid = si.ne(-1)
    layout = torch.tensor(clib.inverse_cdf_layout(n), dtype=torch.int64)
    stream = ext.ctypes_stream(cuda)
    count = torch.empty(n, dtype=torch.int32, device=cuda)
    check(LIB.nsvf_sample_count(n, H, I.data_ptr(), L.data_ptr(), Hh.data_ptr(), probs.data_ptr(),
                                steps.data_ptr(), layout.data_ptr(), count.data_ptr(), stream),
          "sample_count")
    assert torch.equal(count.long(), valid.sum(1))
    offset = torch.zeros(n + 1, dtype=torch.int64, device=cuda)
    torch.cumsum(count, 0, out=offset[1:])
    ns = int(offset[-1].item())
    vox = torch.empty(ns, dtype=torch.int32, device=cuda)
    xyzd = torch.empty(ns, 4, device=cuda)
    depth = torch.empty(ns, device=cuda)
    err = ext.error_word(cuda)
    check(LIB.nsvf_sample_compact(n, H, I.data_ptr(), L.data_ptr(), Hh.data_ptr(),
                                  probs.data_ptr(), steps.data_ptr(), layout.data_ptr(),
                                  ro.data_ptr(), 3, rd.data_ptr(), offset.data_ptr(),
                                  vox.data_ptr(), xyzd.data_ptr(), depth.data_ptr(),
                                  err.data_ptr(), stream), "sample_compact")
    ext.check_errors(cuda)
    assert ns == int(valid.sum()) > 1000
    assert torch.equal(vox, si[valid].int())
    assert torch.equal(depth, sd[valid])
    assert torch.equal(xyzd[:, 3], ss[valid].clamp(min=0))
    row = torch.arange(n, device=cuda)[:, None].expand_as(si)[valid]
    xyz = ro[row] + rd[row] * sd[valid][:, None]
    assert torch.equal(xyzd[:, :3], xyz)
