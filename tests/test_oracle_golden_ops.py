"""The CPU oracle against the fixtures of tests/golden/make_golden_ops.py
(made by running the reference itself): the parallel uniform sampler, the
uniform op wrapper, ball intersection and a 6,000-ray subset of the 800x800
c2 frame (raw SVO, sorted lists, inverse-CDF samples given the reference's
distribution). This pins the oracle beyond the 147-voxel scene."""
import numpy as np

from oracle import cpu


def _c1(golden):
    hit = golden["svo_hits"][0]
    return (golden["svo_intersected_voxel_idx"][0][hit], golden["svo_min_depth"][0][hit],
            golden["svo_max_depth"][0][hit])


def _par_agrees(out, go, tag, I, L, U):
    si, sd, ss = out
    assert np.array_equal(sd, go["%s_depth" % tag]) and np.array_equal(ss, go["%s_dists" % tag])
    return cpu.shared_face_ids_agree(si, go["%s_idx" % tag], sd, ss, I, L, U)


def test_parallel_sampler(golden, golden_ops):
    """Depths and distances bit for bit; ids bit for bit except after faces
    shared by two voxels, where the reference's sort order is unspecified."""
    go = golden_ops
    I, L, U = _c1(golden)
    march = float(go["par_march"])
    n = _par_agrees(cpu.parallel_ray_sampling(march, I, L, U), go, "par_det", I, L, U)
    n += _par_agrees(cpu.parallel_ray_sampling(march, I, L, U, go["par_noise"]), go, "par_rand",
                     I, L, U)
    assert n > 0


def test_parallel_sampler_c2_chunks(golden_ops):
    go = golden_ops
    h = go["c2_hits"].reshape(-1)
    I = go["c2_intersected_voxel_idx"].reshape(h.size, -1)[h]
    L = go["c2_min_depth"].reshape(h.size, -1)[h]
    U = go["c2_max_depth"].reshape(h.size, -1)[h]
    parts = [cpu.parallel_ray_sampling(1.0 / 512, I[i:i + 4096], L[i:i + 4096], U[i:i + 4096])
             for i in range(0, I.shape[0], 4096)]
    assert len(parts) == 2
    W = max(p[0].shape[1] for p in parts)
    out = [np.concatenate([np.pad(p[j], ((0, 0), (0, W - p[j].shape[1])), constant_values=pad)
                           for p in parts]) for j, pad in enumerate([-1, 10000.0, 0.0])]
    _par_agrees(out, go, "c2_par", I, L, U)


def test_uniform_wrapper(golden, golden_ops):
    go = golden_ops
    I, L, U = _c1(golden)
    N, P = I.shape
    march = np.float32(go["par_march"])
    steps = int(float(go["uni_max_len"]) / float(march)) + 2 * P
    Hp = int(np.ceil(N / 256)) * 256
    cat = lambda x: np.concatenate([x, x[:Hp - N]], 0).reshape(256, -1, P)
    for noise, tag in [(np.full((Hp, steps), 0.5, np.float32), "det"), (go["uni_noise"], "rand")]:
        si, sd, ss = cpu.uniform_ray_sampling(cat(I), cat(L), cat(U), noise.reshape(256, -1, steps),
                                              float(march), steps)
        si, sd, ss = (x.reshape(Hp, -1)[:N] for x in (si, sd, ss))
        w = int((si != -1).sum(-1).max())
        for got, k in zip([si[:, :w], sd[:, :w], ss[:, :w]], ["idx", "depth", "dists"]):
            assert np.array_equal(got, go["uni_%s_%s" % (tag, k)]), (tag, k)


def test_ball(golden, golden_ops):
    go = golden_ops
    R = golden["ray_dir"].shape[0]
    rs = np.broadcast_to(golden["ray_start"], (R, 3))[None]
    idx, lo, hi = cpu.ball_intersect(rs, golden["ray_dir"][None], golden["points"][None],
                                     float(go["ball_radius"]), 20)
    assert np.array_equal(idx, go["ball_idx"])
    np.testing.assert_allclose(lo, go["ball_min"], atol=3e-4)
    np.testing.assert_allclose(hi, go["ball_max"], atol=3e-4)


def test_c2_subset(golden_ops):
    go = golden_ops
    R = go["c2_ray_dir"].shape[0]
    rs = np.broadcast_to(go["c2_ray_start"], (R, 3))[None]
    raw = cpu.svo_intersect(rs, go["c2_ray_dir"][None], go["c2_octree_centers"][None],
                            go["c2_octree_children"][None], 1.0 / 64, 64)
    for got, k in zip(raw, ["idx", "min", "max"]):
        assert np.array_equal(got, go["c2_raw_%s" % k]), k
    idx, lo, hi = cpu.sort_hits(*raw)
    assert np.array_equal(lo, go["c2_min_depth"]) and np.array_equal(hi, go["c2_max_depth"])
    assert np.array_equal(idx, go["c2_intersected_voxel_idx"])
    h = go["c2_hits"].reshape(-1)
    assert np.array_equal((idx[0] != -1).any(-1), h)
    I, L, U = idx[0][h], lo[0][h], hi[0][h]
    pr, st = cpu.probs_steps(I, L, U, 1.0 / 512)
    ref_st = go["c2_steps"].reshape(-1)[h]
    np.testing.assert_allclose(st, ref_st, rtol=3e-7)
    N = I.shape[0]
    ref_pr = go["c2_probs"].reshape(-1, 64)[h]
    M = int(np.ceil(ref_st).max()) + 64
    si, sd, ss = cpu.inverse_cdf_op(I, L, U, ref_pr, ref_st, np.full((N, M), 0.5, np.float32))
    ref_si = go["c2_det_sampled_point_voxel_idx"]
    assert np.array_equal(si, ref_si)
    m = ref_si != -1
    assert np.array_equal(sd[m], go["c2_det_sampled_point_depth"][m])
    assert np.array_equal(np.maximum(ss[m], 0), go["c2_det_sampled_point_distance"][m])


def test_hierarchical_resampling(golden, golden_hier):
    """The oracle's fine-pass inputs and fine samples against the reference's
    (golden_hier.npz): bit for bit, except the normalised probabilities
    (torch's pairwise sum, ~1e-6 relative); fine samples from the reference's
    inputs."""
    g, gh = golden, golden_hier
    for tag, kw in [("nerf64", dict(fixed_fine_num_samples=64)),
                    ("nsvf2", dict(fine_num_sample_ratio=2.0))]:
        lo, hi, vid, pr, st = cpu.prepare_hierarchical(
            g["svo_det_sampled_point_depth"], g["svo_det_sampled_point_distance"],
            g["svo_det_sampled_point_voxel_idx"], g["render_probs"], **kw)
        assert np.array_equal(lo, gh["%s_min_depth" % tag])
        assert np.array_equal(hi, gh["%s_max_depth" % tag])
        assert np.array_equal(vid, gh["%s_intersected_voxel_idx" % tag])
        assert np.array_equal(st, gh["%s_steps" % tag])
        # a sequential sum adds the ~1e-5 padding terms onto ~1 one by one; torch's
        # pairwise sum keeps them apart: ~1e-6 relative
        np.testing.assert_allclose(pr, gh["%s_probs" % tag], rtol=5e-6, atol=0)
        I, L, U = (gh["%s_%s" % (tag, k)] for k in ["intersected_voxel_idx", "min_depth", "max_depth"])
        P, S = gh["%s_probs" % tag], gh["%s_steps" % tag]
        N, Hh = I.shape
        M = int(np.ceil(S).max()) + Hh
        si, sd, ss = cpu.inverse_cdf_op(I, L, U, P, S, np.full((N, M), 0.5, np.float32))
        ref = gh["%s_fine_sampled_point_voxel_idx" % tag]
        assert np.array_equal(si, ref)
        m = ref != -1
        assert np.array_equal(sd[m], gh["%s_fine_sampled_point_depth" % tag][m])
        assert np.array_equal(np.maximum(ss[m], 0), gh["%s_fine_sampled_point_distance" % tag][m])
