"""The GPU ops against fixtures made by running the reference itself
(tests/golden/make_golden_ops.py -> golden_ops.npz):

* the back-up parallel uniform sampler (clib.parallel_ray_sampling, the
  nsvf_parallel_ray_sampling kernel): deterministic and recorded-jitter
  outputs on the 147-voxel scene, and two 4,096-ray chunks of the c2 frame;
* the UniformRaySampling wrapper and op (deterministic / recorded noise);
* ball intersection;
* a 6,000-ray subset of the 800x800 c2 frame: raw SVO outputs, the sorted
  lists and hit flags, the sampling distribution, and the inverse-CDF
  samples -- bit for bit except the distribution, whose per-ray sum the
  reference takes in torch's reduction order (1 ulp)."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _t(a, dev):
    return torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def _c1_lists(golden, dev):
    hit = golden["svo_hits"][0]
    return (_t(golden["svo_intersected_voxel_idx"][0][hit], dev),
            _t(golden["svo_min_depth"][0][hit], dev), _t(golden["svo_max_depth"][0][hit], dev))


def _eq(got, ref):
    got = got.cpu().numpy() if isinstance(got, torch.Tensor) else got
    assert got.shape == ref.shape, (got.shape, ref.shape)
    assert np.array_equal(got, ref)


def _par_check(out, go, tag, I, L, U):
    """Depths and distances bit for bit; ids bit for bit except after faces
    shared by two voxels, where the reference's torch.sort order is
    unspecified (there: one of the two voxels, oracle.cpu's checker); and
    equal to the oracle's restatement (same tie rule) everywhere."""
    from oracle import cpu
    si, sd, ss = (x.cpu().numpy() for x in out)
    assert np.array_equal(sd, go["%s_depth" % tag]) and np.array_equal(ss, go["%s_dists" % tag])
    I, L, U = (x.cpu().numpy() for x in (I, L, U))
    cpu.shared_face_ids_agree(si, go["%s_idx" % tag], sd, ss, I, L, U)
    return si


def test_parallel_sampling_matches_reference(golden, golden_ops, cuda):
    from nsvf_gb300 import clib, ext
    from oracle import cpu
    go = golden_ops
    I, L, U = _c1_lists(golden, cuda)
    march = float(go["par_march"])
    si = _par_check(clib.parallel_ray_sampling(march, I, L, U, True), go, "par_det", I, L, U)
    assert np.array_equal(si, cpu.parallel_ray_sampling(march, *(x.cpu().numpy() for x in (I, L, U)))[0])
    # recorded jitter through the op
    noise = _t(go["par_noise"], cuda)
    n, K = noise.shape
    H = I.shape[1]
    W = 2 * H + K - 1
    si = torch.empty(n, W, dtype=torch.int32, device=cuda)
    sd, ss = torch.empty(n, W, device=cuda), torch.empty(n, W, device=cuda)
    cnt = torch.zeros(n, dtype=torch.int32, device=cuda)
    ext.parallel_ray_sampling_rows(I.int().contiguous(), L, U, noise, march, K, si, sd, ss, cnt)
    w = int(cnt.max())
    _par_check((si[:, :w], sd[:, :w], ss[:, :w]), go, "par_rand", I, L, U)


def test_parallel_sampling_chunks_match_reference_c2(golden_ops, cuda):
    from nsvf_gb300 import clib
    go = golden_ops
    h = go["c2_hits"].reshape(-1)
    I = _t(go["c2_intersected_voxel_idx"].reshape(h.size, -1)[h], cuda)
    L = _t(go["c2_min_depth"].reshape(h.size, -1)[h], cuda)
    U = _t(go["c2_max_depth"].reshape(h.size, -1)[h], cuda)
    assert I.shape[0] > 4096
    _par_check(clib.parallel_ray_sampling(1.0 / 512, I, L, U, True), go, "c2_par", I, L, U)


def test_uniform_sampling_matches_reference(golden, golden_ops, cuda):
    from nsvf_gb300 import clib, ext
    go = golden_ops
    I, L, U = _c1_lists(golden, cuda)
    march = float(go["par_march"])
    max_len = float(go["uni_max_len"])
    out = clib.uniform_ray_sampling(I, L, U, march, max_len, True)
    for got, k in zip(out, ["idx", "depth", "dists"]):
        _eq(got, go["uni_det_%s" % k])
    # recorded noise through the op, on the wrapper's 256-block padded layout
    N, P = I.shape
    Hp = int(np.ceil(N / 256)) * 256
    cat = lambda x: torch.cat([x, x[:Hp - N]], 0).reshape(256, -1, P).contiguous()
    noise = _t(go["uni_noise"], cuda).reshape(256, Hp // 256, -1).contiguous()
    si, sd, ss = ext.uniform_ray_sampling(cat(I.int()), cat(L), cat(U), noise, march,
                                          noise.shape[-1])
    si, sd, ss = (x.reshape(Hp, -1)[:N] for x in (si, sd, ss))
    w = int(si.ne(-1).sum(-1).max())
    for got, k in zip([si[:, :w], sd[:, :w], ss[:, :w]], ["idx", "depth", "dists"]):
        _eq(got, go["uni_rand_%s" % k])


def test_ball_intersect_matches_reference(golden, golden_ops, cuda):
    """Ids and hit order bit for bit; depths to 3e-4 (the reference squares
    with pow, this library with a multiplication)."""
    from nsvf_gb300 import ext
    go = golden_ops
    R = golden["ray_dir"].shape[0]
    rs = _t(np.broadcast_to(golden["ray_start"], (R, 3)), cuda)[None]
    rd = _t(golden["ray_dir"], cuda)[None]
    pts = _t(golden["points"], cuda)[None]
    idx, lo, hi = ext.ball_intersect(rs, rd, pts, float(go["ball_radius"]), 20)
    _eq(idx, go["ball_idx"])
    assert int((idx != -1).sum()) > 1000
    np.testing.assert_allclose(lo.cpu().numpy(), go["ball_min"], atol=3e-4)
    np.testing.assert_allclose(hi.cpu().numpy(), go["ball_max"], atol=3e-4)


def test_c2_subset_matches_reference(golden_ops, cuda):
    from nsvf_gb300 import clib, ext
    go = golden_ops
    R = go["c2_ray_dir"].shape[0]
    o = _t(np.broadcast_to(go["c2_ray_start"], (R, 3)), cuda)[None]
    d = _t(go["c2_ray_dir"], cuda)[None]
    cen = _t(go["c2_octree_centers"], cuda)[None]
    chi = _t(go["c2_octree_children"], cuda)[None]
    raw = ext.svo_intersect(o, d, cen, chi, 1.0 / 64, 64)
    for got, k in zip(raw, ["idx", "min", "max"]):
        _eq(got, go["c2_raw_%s" % k])
    idx, lo, hi, hits = ext.svo_intersect_sorted(o, d, cen, chi, 1.0 / 64, 64)
    _eq(idx, go["c2_intersected_voxel_idx"])
    _eq(lo, go["c2_min_depth"])
    _eq(hi, go["c2_max_depth"])
    _eq(hits.bool(), go["c2_hits"])
    h = torch.from_numpy(go["c2_hits"].reshape(-1)).to(cuda)
    assert int(h.sum()) > 4096
    # the distribution: slot-order sum vs torch's reduction order
    probs, steps = ext.ray_probs(idx[0][h], lo[0][h], hi[0][h], 1.0 / 512)
    ref_steps = go["c2_steps"].reshape(-1)[go["c2_hits"].reshape(-1)]
    np.testing.assert_allclose(steps.cpu().numpy(), ref_steps, rtol=3e-7)
    # inverse-CDF placement given the reference's distribution, bit for bit
    pr = _t(go["c2_probs"].reshape(-1, 64)[go["c2_hits"].reshape(-1)], cuda)
    st = _t(ref_steps, cuda)
    out = clib.inverse_cdf_sampling(idx[0][h].contiguous(), lo[0][h].contiguous(),
                                    hi[0][h].contiguous(), pr, st, -1, True)
    for got, k in zip(out, ["sampled_point_voxel_idx", "sampled_point_depth",
                            "sampled_point_distance"]):
        ref = go["c2_det_%s" % k]
        if k != "sampled_point_voxel_idx":
            # the encoder's post-processing (MAX_DEPTH / 0 where the id is -1, dists >= 0)
            m = go["c2_det_sampled_point_voxel_idx"] != -1
            got = got.cpu().numpy()
            assert np.array_equal(got[m] if k == "sampled_point_depth" else np.maximum(got[m], 0),
                                  ref[m])
        else:
            _eq(got, ref)
