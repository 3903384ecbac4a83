"""The C oracle (oracle/clib_oracle.c) against the reference's own kernel
bodies compiled for the CPU (oracle/_ref, built by oracle/build_ref.py) on
the c2 workload: the 125,476-voxel shell, rays of the 800x800 frame 0.

* SVO traversal on 20,000 seeded rays and AABB intersection on 300, bit for
  bit; ball intersection on 300, with decisions allowed to differ only for
  balls within FP32 rounding of the radius, and depths by that rounding;
* uniform sampling on the wrapper's 256-block layout with seeded noise;
* inverse-CDF sampling through the reference's InverseCDFRaySampling wrapper
  (200 blocks, launched 800 columns at a time; deterministic and seeded) on
  200,000 hit lists (the frame's hit rays repeated, so that the 800-column
  slicing and the cross-row reads it decides are exercised).

Runs only where the reference checkout exists (it compiles the reference's
sources); skipped elsewhere."""
import numpy as np
import pytest
import torch

from oracle import build_ref, cpu, workload

pytestmark = pytest.mark.skipif(not build_ref.available(), reason="reference checkout absent")


@pytest.fixture(scope="module")
def c2():
    build_ref.build_clib()
    sc = workload.c2_scene()
    rs, rd = workload.frame(0)
    return sc, rs, rd


def _rays(rs, rd, n, seed):
    sel = np.sort(np.random.RandomState(seed).choice(rd.shape[0], n, replace=False))
    return np.broadcast_to(rs, (n, 3))[None].copy(), rd[sel][None].copy()


def test_svo_aabb_ball_at_c2_scale(c2):
    from oracle import ref_clib
    sc, rs, rd = c2
    vs = sc["voxel_size"]
    cen, chi = sc["octree"]
    o, d = _rays(rs, rd, 20000, 1)
    a = cpu.svo_intersect(o, d, cen[None], chi[None], vs, 64)
    b = ref_clib.svo_intersect(o, d, cen[None], chi[None], vs, 64)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert (a[0] != -1).any(-1).sum() > 2000
    o, d = _rays(rs, rd, 300, 2)
    pts = sc["centers_shifted"][None]
    a = cpu.aabb_intersect(o, d, pts, vs, 64)
    b = ref_clib.aabb_intersect(o, d, pts, vs, 64)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    rad = vs * 0.6
    a = cpu.ball_intersect(o, d, pts, rad, 64)
    b = ref_clib.ball_intersect(o, d, pts, rad, 64)
    assert (a[0] != -1).sum() > 100
    # The ball test r2 = |x|^2 - (d.x)^2 < radius^2 cancels ~16 against
    # ~1e-4 at distance 4, so the FMA contraction the compiler picks flips
    # balls within FP32 rounding of the radius. Every other decision, and the
    # depths of the balls both keep, agree.
    P = pts[0].astype(np.float64)
    for r in range(o.shape[1]):
        sa = set(a[0][0, r][a[0][0, r] != -1].tolist())
        sb = set(b[0][0, r][b[0][0, r] != -1].tolist())
        for k in sa ^ sb:
            x = P[k] - o[0, r].astype(np.float64)
            dd = d[0, r].astype(np.float64)
            r2 = x @ x - (x @ dd) ** 2
            assert abs(r2 - rad * rad) <= 4e-6 * (x @ x), (r, k, r2, rad * rad)
        for k in sa & sb:
            # depth -/+ sqrt(radius^2 - r2): the same rounding of r2, divided
            # by 2 sqrt(radius^2 - r2) (at most its square root near tangency)
            x = P[k] - o[0, r].astype(np.float64)
            dd = d[0, r].astype(np.float64)
            slack = rad * rad - (x @ x - (x @ dd) ** 2)
            e = 4e-6 * (x @ x)
            tol = 3e-4 + min(e / (2 * np.sqrt(max(slack, 0.0)) + 1e-30), np.sqrt(e))
            ia = list(a[0][0, r]).index(k)
            ib = list(b[0][0, r]).index(k)
            assert abs(a[1][0, r, ia] - b[1][0, r, ib]) <= tol
            assert abs(a[2][0, r, ia] - b[2][0, r, ib]) <= tol


def _hit_lists(c2, n_rays=40000):
    sc, rs, rd = c2
    cen, chi = sc["octree"]
    o, d = _rays(rs, rd, n_rays, 3)
    idx, lo, hi = cpu.sort_hits(*cpu.svo_intersect(o, d, cen[None], chi[None], sc["voxel_size"],
                                                   64))
    h = (idx[0] != -1).any(-1)
    return idx[0][h], lo[0][h], hi[0][h]


def test_uniform_at_c2_scale(c2):
    from oracle import ref_clib
    I, L, U = _hit_lists(c2)
    N, P = I.shape
    step = np.float32(1.0 / 512)
    steps = int(2.0 / float(step)) + 2 * P
    Hp = int(np.ceil(N / 256)) * 256
    cat = lambda x: np.concatenate([x, x[:Hp - N]], 0).reshape(256, -1, P)
    noise = np.random.RandomState(4).rand(256, Hp // 256, steps).astype(np.float32)
    a = cpu.uniform_ray_sampling(cat(I), cat(L), cat(U), noise, float(step), steps)
    b = ref_clib.uniform_ray_sampling(cat(I), cat(L), cat(U), noise, float(step), steps)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    assert (a[0] != -1).sum() > 100000


def test_inverse_cdf_wrapper_layout_at_c2_scale(c2):
    from oracle import ref_import
    ref = ref_import.load()
    I, L, U = _hit_lists(c2)
    reps = -(-200000 // I.shape[0])
    I, L, U = (np.concatenate([x] * reps)[:200000] for x in (I, L, U))
    pr, st = cpu.probs_steps(I, L, U, 1.0 / 512)
    N, P = I.shape
    K = -(-N // 200)
    assert K > 800                       # two column launches per block
    M = int(np.ceil(st).max()) + P
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x))
    # deterministic
    out = ref.clib.inverse_cdf_sampling(t(I), t(L), t(U), t(pr), t(st), -1, True)
    mine = cpu.inverse_cdf_op(I, L, U, pr, st, np.full((N, M), 0.5, np.float32))
    for x, y in zip(mine, out):
        assert np.array_equal(x, y.numpy())
    # seeded noise: the wrapper draws [200 * K, M] U(0, 1) clamped to [.001, .999]
    torch.manual_seed(9)
    noise = torch.zeros(200 * K, M).uniform_().clamp(min=0.001, max=0.999).numpy()
    torch.manual_seed(9)
    out = ref.clib.inverse_cdf_sampling(t(I), t(L), t(U), t(pr), t(st), -1, False)
    mine = cpu.inverse_cdf_op(I, L, U, pr, st, noise)
    for x, y in zip(mine, out):
        assert np.array_equal(x, y.numpy())
