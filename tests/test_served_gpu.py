"""The served renderer (compacted samples, tcgen05 BF16 MLP, compensated
compositing) against the drop-in FP32 path and the float64 oracle.

The geometry is shared: both paths build each ray's sampling distribution
with the same slot-order sum (nsvf_ray_probs / nsvf_gather_probs, pinned bit
for bit below), so the served path evaluates exactly the drop-in path's
samples: same voxel ids, depths and distances, bit for bit, also on the full
800x800 c2 frame. Colours: BF16 field vs the FP32 render within 2e-3 max abs
RGB error, the workload's bar."""
import argparse

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _scene(dev, voxel, embed_std, sigma_scale, sigma_bias, max_hits):
    from nsvf_gb300 import scenes
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.renderer import VolumeRenderer
    if voxel == 0.25:
        p, vs = scenes.scene_small()
    else:
        p, vs = scenes.scene_shell(voxel)
    args = argparse.Namespace(voxel_size=vs, max_hits=max_hits, raymarching_stepsize_ratio=0.125,
                              voxel_embed_dim=32, use_octree=True, deterministic_step=True,
                              chunk_size=64)
    enc = SparseVoxelEncoder(args, points=p)
    with torch.no_grad():
        enc.values.weight.copy_(scenes.voxel_embeddings(enc.values.weight.shape[0], 32,
                                                        embed_std, seed=1))
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=2, sigma_scale=sigma_scale,
                                                             sigma_bias=sigma_bias))
    return enc.to(dev).eval(), field.to(dev).eval(), VolumeRenderer(args).eval(), vs


@pytest.mark.parametrize("voxel,size,std,ss,sb,H", [
    (0.25, 64, 1.0, 60.0, 0.5, 20),          # small scene, opaque field
    (1.0 / 32, 160, 1.0, 30.0, 0.5, 64),     # shell scene
    (1.0 / 32, 160, 0.01, 1.0, 0.0, 64),     # the workloads' near-transparent init
])
def test_served_matches_dropin(cuda, voxel, size, std, ss, sb, H):
    from nsvf_gb300 import ext, scenes
    from nsvf_gb300.renderer import render_rays
    from nsvf_gb300.served import SceneState, render_frame
    enc, field, ren, vs = _scene(cuda, voxel, std, ss, sb, H)
    rs, rd = scenes.pinhole_rays(scenes.sphere_cameras(3, 4.0, seed=9)[1], size, size,
                                 80.0 * size / 64.0)
    rs_t = torch.from_numpy(rs).to(cuda)
    rd_t = torch.from_numpy(rd).to(cuda)
    with torch.no_grad():
        ref = render_rays(enc, field, ren, rs_t.reshape(1, 1, 1, 3), rd_t.reshape(1, 1, -1, 3))
    scene = SceneState(enc, field)
    rcol = ref["colors"].reshape(-1, 3).cpu().numpy()
    # 1) the served chain with the FP32 field equals the drop-in FP32 path
    #    (without the double-float pass, which the drop-in path does not have)
    f32 = render_frame(scene, rs_t, rd_t, mlp="fp32", kahan=False, exact=False)
    np.testing.assert_allclose(f32["colors"].cpu().numpy(), rcol, atol=2e-5)
    np.testing.assert_allclose(f32["missed"].cpu().numpy(), ref["missed"].reshape(-1).cpu().numpy(),
                               atol=2e-5)
    np.testing.assert_allclose(f32["depths"].cpu().numpy(), ref["depths"].reshape(-1).cpu().numpy(),
                               rtol=1e-5, atol=1e-4)
    # 2) the tensor-core MLP equals its torch emulation inside the chain; with
    #    the opaque test fields a BF16 rounding tie that the two accumulation
    #    orders break differently moves a pixel by a few 1e-3
    out = render_frame(scene, rs_t, rd_t)
    emu = render_frame(scene, rs_t, rd_t, mlp="bf16_emulated")
    ext.check_errors(cuda)
    col = out["colors"].cpu().numpy()
    np.testing.assert_allclose(col, emu["colors"].cpu().numpy(), atol=2e-3 if ss == 1.0 else 8e-3)
    # 3) BF16 vs FP32: within the workload bar (2e-3) for the workload's
    #    near-transparent field; the opaque test fields (sigma scaled 30-60x)
    #    amplify the BF16 rounding of sigma and get a wider bound
    err = np.abs(col - rcol).max()
    assert err <= (2e-3 if ss == 1.0 else 8e-2), err
    # exactly the drop-in path's samples
    smp = _dropin_samples(enc, rs_t, rd_t)
    assert out["n_samples"] == int(smp['sampled_point_voxel_idx'].ne(-1).sum())
    assert out["n_hit_rays"] == smp["n_hit"]


def _dropin_samples(enc, rs_t, rd_t):
    """The drop-in path's samples of a frame: intersection, nsvf_ray_probs,
    the reference wrapper's inverse-CDF sampling (deterministic jitter)."""
    from nsvf_gb300 import ext
    with torch.no_grad():
        st = enc.precompute(id=None)
        _, _, inter, hits = enc.ray_intersect(rs_t.reshape(1, 1, 1, 3), rd_t.reshape(1, 1, -1, 3),
                                              {k: (v.unsqueeze(0) if v is not None else None)
                                               for k, v in st.items()})
        inter['probs'], inter['steps'] = ext.ray_probs(inter['intersected_voxel_idx'],
                                                       inter['min_depth'], inter['max_depth'],
                                                       enc.step_size)
        sub = {k: v[hits] for k, v in inter.items()}
        smp = enc.ray_sample(sub)
    smp["n_hit"] = int(hits.sum())
    return smp


def test_served_samples_equal_dropin_c2_frame(cuda):
    """The full 800x800 c2 frame (125,476-voxel shell, max_hits 64, step
    1/512): the served chain's compacted samples are the drop-in path's valid
    samples in ray order, voxel ids, depths and distances equal bit for bit
    (zero tolerance)."""
    from nsvf_gb300 import ext, scenes, served
    enc, field, ren, vs = _scene(cuda, 1.0 / 64, 0.01, 1.0, 0.0, 64)
    rs, rd = scenes.frame_view(0, size=800)
    rs_t, rd_t = torch.from_numpy(rs).to(cuda), torch.from_numpy(rd).to(cuda)
    scene = served.SceneState(enc, field)
    out = served.render_frame(scene, rs_t, rd_t)
    ext.check_errors(cuda)
    b = next(iter(scene._frames.values()))
    ns = out["n_samples"]
    smp = _dropin_samples(enc, rs_t, rd_t)
    vid = smp['sampled_point_voxel_idx']
    mask = vid.ne(-1)
    assert out["n_hit_rays"] == smp["n_hit"] > 100000
    assert ns == int(mask.sum()) > 10 ** 7
    assert torch.equal(b["vox"][:ns], vid[mask].int())
    assert torch.equal(b["depth"][:ns], smp['sampled_point_depth'][mask])
    assert torch.equal(b["xyzd"][:ns, 3], smp['sampled_point_distance'][mask])


@pytest.mark.parametrize("H", [20, 64, 100])
def test_probs_slot_order(cuda, H):
    """nsvf_gather_probs and nsvf_ray_probs, bit for bit: d = max - min on hit
    slots, tot = d_0 + d_1 + ... one slot at a time in slot order (FP32),
    probs = d / tot, steps = tot / step; the oracle's probs_steps is the same
    sequential sum. gather_probs reads a row up to its first -1 and pads its
    copy like the traversals pad their rows (depths 10000)."""
    from nsvf_gb300 import ext
    from nsvf_gb300._lib import LIB
    from oracle import cpu
    rng = np.random.RandomState(H)
    R, step = 700, np.float32(1.0 / 256)
    idx = rng.randint(0, 5000, (R, H)).astype(np.int32)
    m = rng.randint(0, H + 1, R)
    idx[np.arange(H)[None, :] >= m[:, None]] = -1
    lo = (rng.rand(R, H) * 4).astype(np.float32)
    hi = (lo + rng.rand(R, H).astype(np.float32) * np.float32(0.05)).astype(np.float32)
    pix = np.nonzero(m > 0)[0].astype(np.int64)
    n = pix.size
    d = np.where(idx[pix] == -1, np.float32(0), hi[pix] - lo[pix]).astype(np.float32)
    tot = np.zeros((n, 1), np.float32)
    for k in range(H):
        tot[:, 0] = tot[:, 0] + d[:, k]
    o_probs, o_steps = cpu.probs_steps(idx[pix], lo[pix], hi[pix], step)
    assert np.array_equal(o_steps, tot[:, 0] / step)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(cuda)
    pr_all, st_all = ext.ray_probs(t(idx), t(lo), t(hi), float(step))
    assert np.array_equal(pr_all.cpu().numpy()[pix], d / tot)
    assert np.array_equal(st_all.cpu().numpy()[pix], tot[:, 0] / step)
    assert np.array_equal(pr_all.cpu().numpy()[pix], o_probs)
    I = torch.empty(R, H, dtype=torch.int32, device=cuda)
    L, U, probs = (torch.empty(R, H, device=cuda) for _ in range(3))
    steps = torch.empty(R, device=cuda)
    pix_d, idx_d, lo_d, hi_d = t(pix), t(idx), t(lo), t(hi)
    n_d = torch.tensor([n], dtype=torch.int64, device=cuda)
    assert LIB.nsvf_gather_probs(R, n_d.data_ptr(), H, float(step), pix_d.data_ptr(), idx_d.data_ptr(),
                                 lo_d.data_ptr(), hi_d.data_ptr(), I.data_ptr(), L.data_ptr(),
                                 U.data_ptr(), probs.data_ptr(), steps.data_ptr(),
                                 ext.ctypes_stream(cuda)) == 0
    assert np.array_equal(I[:n].cpu().numpy(), idx[pix])
    # slots past a row's first -1 are copied as the traversals pad them
    pad = idx[pix] == -1
    assert np.array_equal(L[:n].cpu().numpy(), np.where(pad, np.float32(10000), lo[pix]))
    assert np.array_equal(U[:n].cpu().numpy(), np.where(pad, np.float32(10000), hi[pix]))
    assert np.array_equal(probs[:n].cpu().numpy(), d / tot)
    assert np.array_equal(steps[:n].cpu().numpy(), tot[:, 0] / step)


@pytest.mark.parametrize("std,ss,sb,max_err,rms_err", [
    (0.01, 1.0, 0.0, 2e-3, 5e-4),     # the workloads' field: the 2e-3 bar
    (1.0, 60.0, 0.5, 8e-2, 1e-2),     # opaque test field: BF16 sigma rounding amplified
])
def test_served_vs_float64_oracle(cuda, std, ss, sb, max_err, rms_err):
    """Max and RMS RGB error of the served BF16 frame against a float64 render
    of the same samples (oracle), small scene."""
    from nsvf_gb300 import scenes
    from nsvf_gb300.served import SceneState, render_frame
    from oracle import cpu
    enc, field, ren, vs = _scene(cuda, 0.25, std, ss, sb, 20)
    rs, rd = scenes.small_view(0)
    scene = SceneState(enc, field)
    out = render_frame(scene, torch.from_numpy(rs).to(cuda), torch.from_numpy(rd).to(cuda))
    col = out["colors"].cpu().numpy()
    # float64 oracle on the same rays
    st = enc.precompute(id=None)
    cen, chi = st['voxel_octree_center_xyz'].cpu().numpy(), st['voxel_octree_children_idx'].cpu().numpy()
    R = rd.shape[0]
    idx, lo, hi = cpu.sort_hits(*cpu.svo_intersect(np.broadcast_to(rs, (R, 3))[None], rd[None],
                                                   cen[None], chi[None], vs, 20))
    idx, lo, hi = idx[0], lo[0], hi[0]
    hit = (idx != -1).any(-1)
    pr, stp = cpu.probs_steps(idx[hit], lo[hit], hi[hit], vs / 8)
    N = int(hit.sum())
    M = int(np.ceil(stp).max()) + 20
    si, sd, ss = cpu.inverse_cdf_op(idx[hit], lo[hit], hi[hit], pr, stp, np.full((N, M), 0.5, np.float32))
    ss = np.maximum(ss, 0)
    mask = si != -1
    xyz = rs[None, None].astype(np.float64) + rd[hit][:, None].astype(np.float64) * sd[..., None]
    emb = cpu.trilinear_embed(xyz[mask], si[mask], st['voxel_center_xyz'].cpu().numpy(),
                              st['voxel_vertex_idx'].cpu().numpy(),
                              st['voxel_vertex_emb'].detach().cpu().numpy(), vs)
    W = [(l.weight.detach().cpu().numpy(), l.bias.detach().cpu().numpy()) for l in field.layers]
    sig, rgb = cpu.mlp_forward(emb, W)
    S = np.zeros(mask.shape)
    C = np.zeros(mask.shape + (3,))
    S[mask], C[mask] = sig, rgb
    o = cpu.composite(S, C, sd.astype(np.float64), ss.astype(np.float64), mask)
    ref = np.ones((R, 3))
    ref[hit] = o["colors"] + o["missed"][:, None]
    err = np.abs(col - ref)
    assert err.max() <= max_err, err.max()
    assert np.sqrt((err ** 2).mean()) <= rms_err


def test_sample_capacity_overflow_is_rendered_again(cuda, monkeypatch):
    """A frame with more samples than the sample buffers hold (error bit 1
    from the compaction and the MLP) is composited again with room for all
    of them: the result equals a render whose buffers were large enough."""
    from nsvf_gb300 import ext, scenes, served
    enc, field, ren, vs = _scene(cuda, 1.0 / 32, 1.0, 30.0, 0.5, 64)
    rs, rd = scenes.pinhole_rays(scenes.sphere_cameras(3, 4.0, seed=9)[1], 96, 96, 120.0)
    rs_t, rd_t = torch.from_numpy(rs).to(cuda), torch.from_numpy(rd).to(cuda)
    ref = served.render_frame(served.SceneState(enc, field), rs_t, rd_t)
    monkeypatch.setattr(served, "INITIAL_SAMPLES_PER_RAY", 1)
    scene = served.SceneState(enc, field)
    out = served.render_frame(scene, rs_t, rd_t)
    ext.check_errors(cuda)
    # the first attempt's buffers (1.25 samples per ray) were too small
    assert out["n_samples"] == ref["n_samples"] > rd.shape[0] * 5 // 4
    assert next(iter(scene._frames.values()))["cap"] >= out["n_samples"]
    assert torch.equal(out["colors"], ref["colors"]) and torch.equal(out["depths"], ref["depths"])
    # the capacity grew to hold the frame: the next frame renders in one go
    again = served.render_frame(scene, rs_t, rd_t)
    assert torch.equal(again["colors"], ref["colors"])


def test_host_frames_match_render_frame(cuda):
    """Frames rendered through served.HostFrames (rays from pinned host
    memory, copies on two streams overlapping the neighbouring frames) equal
    render_frame on device tensors, frame by frame, also when a frame's host
    output slot is reused two frames later."""
    from nsvf_gb300 import ext, scenes, served
    enc, field, ren, vs = _scene(cuda, 1.0 / 32, 1.0, 30.0, 0.5, 64)
    scene = served.SceneState(enc, field)
    size = 96
    cams = scenes.sphere_cameras(5, 4.0, seed=11)
    host, refs = [], []
    for c in cams:
        rs, rd = scenes.pinhole_rays(c, size, size, 120.0)
        rs_h = torch.from_numpy(np.ascontiguousarray(rs)).pin_memory()
        rd_h = torch.from_numpy(np.ascontiguousarray(rd)).pin_memory()
        host.append((rs_h, rd_h))
        r = served.render_frame(scene, rs_h.to(cuda), rd_h.to(cuda))
        refs.append((r["colors"].cpu(), r["depths"].cpu()))
    R = size * size
    outs = [(torch.empty(R, 3).pin_memory(), torch.empty(R).pin_memory()) for _ in cams]
    pipe = served.HostFrames(scene, R)
    pipe.render([(h[0], h[1], o[0], o[1]) for h, o in zip(host, outs)])
    ext.check_errors(cuda)
    for (col, dep), (rc, rdp) in zip(outs, refs):
        assert torch.equal(col, rc) and torch.equal(dep, rdp)
    # two host slots for five frames: each slot holds the last frame copied into it
    ring = [(torch.empty(R, 3).pin_memory(), torch.empty(R).pin_memory()) for _ in range(2)]
    pipe.render([(h[0], h[1]) + ring[i % 2] for i, h in enumerate(host)])
    assert torch.equal(ring[0][0], refs[4][0]) and torch.equal(ring[1][0], refs[3][0])
    assert pipe.n_samples > 0


@pytest.mark.parametrize("pieces", [[0], [0, 5, 1000], [0, 2047, 2048, 4000, 6000]])
def test_scan_compact_pieces_equals_two_pass(cuda, pieces):
    """nsvf_sample_scan_compact_pieces against nsvf_sample_count_pieces, a
    prefix sum and nsvf_sample_compact_pieces on a served frame's hit rows
    cut into pieces (each with the reference's launch layout for its own row
    count, as the serving chunks use them): offsets and samples equal bit for
    bit, including a one-row piece and pieces that end past the rows."""
    from nsvf_gb300 import ext, scenes, served
    from nsvf_gb300._lib import LIB
    enc, field, ren, vs = _scene(cuda, 1.0 / 32, 1.0, 30.0, 0.5, 64)
    rs, rd = scenes.pinhole_rays(scenes.sphere_cameras(3, 4.0, seed=9)[1], 160, 160, 200.0)
    rs_t, rd_t = torch.from_numpy(rs).to(cuda), torch.from_numpy(rd).to(cuda)
    scene = served.SceneState(enc, field)
    served.render_frame(scene, rs_t, rd_t)
    ext.check_errors(cuda)
    b = next(iter(scene._frames.values()))
    R, H = rd.shape[0], scene.max_hits
    n = int(b["n_hit"].item())
    assert n > 5000
    P = len(pieces)
    pr = torch.tensor(pieces + [n], dtype=torch.int64, device=cuda)
    p = served._p
    stream = ext.ctypes_stream(cuda)
    common = (R, p(b["n_hit"]), H, p(b["I"]), p(b["L"]), p(b["U"]), p(b["probs"]), p(b["steps"]),
              p(pr), P)
    rays = (p(b["ro"]), 3, p(rd_t), p(b["pix"]))
    cap = R * 64
    count = torch.zeros(R, dtype=torch.int32, device=cuda)
    o2 = torch.zeros(R + 1, dtype=torch.int64, device=cuda)
    assert LIB.nsvf_sample_count_pieces(*common, p(count), stream) == 0
    torch.cumsum(count, 0, out=o2[1:])
    outs = []
    for one_pass in (False, True):
        vox = torch.full((cap,), -7, dtype=torch.int32, device=cuda)
        xyzd = torch.zeros(cap, 4, device=cuda)
        depth = torch.zeros(cap, device=cuda)
        err = torch.zeros(1, dtype=torch.int32, device=cuda)
        if one_pass:
            off = torch.full((R + 1,), -5, dtype=torch.int64, device=cuda)
            nb = int(LIB.nsvf_sample_scan_bytes(R))
            ws = torch.empty(nb, dtype=torch.uint8, device=cuda)
            assert LIB.nsvf_sample_scan_compact_pieces(*common, *rays, p(off), cap, p(vox), p(xyzd),
                                                       p(depth), p(ws), nb, p(err), stream) == 0
        else:
            off = o2
            assert LIB.nsvf_sample_compact_pieces(*common, *rays, p(off), cap, p(vox), p(xyzd),
                                                  p(depth), p(err), stream) == 0
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        outs.append((off, vox, xyzd, depth))
    (o_a, v_a, x_a, d_a), (o_b, v_b, x_b, d_b) = outs
    tot = int(o_a[R].item())
    assert int(o_b[R].item()) == tot > 10 ** 5
    assert torch.equal(o_a[:n + 1], o_b[:n + 1])
    assert torch.equal(v_a, v_b) and torch.equal(d_a, d_b) and torch.equal(x_a, x_b)


@pytest.mark.parametrize("rows", [0, 1, 13, None])
def test_scan_compact_equals_two_pass(cuda, rows):
    """nsvf_sample_scan_compact_dev (counts, prefix sum and samples in one
    pass with a look-back between blocks) against the count pass, a prefix
    sum and the compaction pass on the hit rows of a served frame: offsets
    and samples equal bit for bit, for 0, 1 and 13 rows (a partial block) and
    all ~20k hit rows; with too small a sample buffer both set error bit 2,
    report the same total and write the same samples up to the capacity."""
    from nsvf_gb300 import ext, scenes, served
    from nsvf_gb300._lib import LIB
    enc, field, ren, vs = _scene(cuda, 1.0 / 32, 1.0, 30.0, 0.5, 64)
    rs, rd = scenes.pinhole_rays(scenes.sphere_cameras(3, 4.0, seed=9)[1], 160, 160, 200.0)
    rs_t, rd_t = torch.from_numpy(rs).to(cuda), torch.from_numpy(rd).to(cuda)
    scene = served.SceneState(enc, field)
    served.render_frame(scene, rs_t, rd_t)
    ext.check_errors(cuda)
    b = next(iter(scene._frames.values()))
    R, H = rd.shape[0], scene.max_hits
    n_all = int(b["n_hit"].item())
    assert n_all > 5000
    n = n_all if rows is None else rows
    n_dev = torch.tensor([n], dtype=torch.int64, device=cuda)
    p = served._p
    stream = ext.ctypes_stream(cuda)
    ro = b["ro"]
    common = (R, p(n_dev), H, p(b["I"]), p(b["L"]), p(b["U"]), p(b["probs"]), p(b["steps"]))
    rays = (p(ro), 3, p(rd_t), p(b["pix"]))

    def two_pass(cap):
        count = torch.zeros(R, dtype=torch.int32, device=cuda)
        off = torch.zeros(R + 1, dtype=torch.int64, device=cuda)
        assert LIB.nsvf_sample_count_dev(*common, p(count), stream) == 0
        torch.cumsum(count, 0, out=off[1:])
        vox = torch.full((cap,), -7, dtype=torch.int32, device=cuda)
        xyzd = torch.zeros(cap, 4, device=cuda)
        depth = torch.zeros(cap, device=cuda)
        err = torch.zeros(1, dtype=torch.int32, device=cuda)
        assert LIB.nsvf_sample_compact_dev(*common, *rays, p(off), cap, p(vox), p(xyzd),
                                           p(depth), p(err), stream) == 0
        return off, vox, xyzd, depth, int(err.item())

    def one_pass(cap):
        off = torch.full((R + 1,), -5, dtype=torch.int64, device=cuda)
        vox = torch.full((cap,), -7, dtype=torch.int32, device=cuda)
        xyzd = torch.zeros(cap, 4, device=cuda)
        depth = torch.zeros(cap, device=cuda)
        err = torch.zeros(1, dtype=torch.int32, device=cuda)
        nb = int(LIB.nsvf_sample_scan_bytes(R))
        ws = torch.empty(nb, dtype=torch.uint8, device=cuda)
        assert LIB.nsvf_sample_scan_compact_dev(*common, *rays, p(off), cap, p(vox), p(xyzd),
                                                p(depth), p(ws), nb, p(err), stream) == 0
        # too small a workspace is refused
        assert LIB.nsvf_sample_scan_compact_dev(*common, *rays, p(off), cap, p(vox), p(xyzd),
                                                p(depth), p(ws), nb - 8, p(err),
                                                stream) == ext.NSVF_ERR_CAPACITY
        return off, vox, xyzd, depth, int(err.item())

    total = int(b["offset"][R].item()) if rows is None else None
    for cap in ([max(total, 1), max(total // 2, 1)] if rows is None else [R * 64]):
        o2, v2, x2, d2, e2 = two_pass(cap)
        o1, v1, x1, d1, e1 = one_pass(cap)
        tot = int(o2[R].item())
        assert int(o1[R].item()) == tot
        assert torch.equal(o1[:n + 1], o2[:n + 1])
        if rows is None:
            assert tot == total
        assert e1 == e2 == (2 if tot > cap else 0)
        k = min(tot, cap)
        assert torch.equal(v1[:k], v2[:k]) and torch.equal(d1[:k], d2[:k])
        assert torch.equal(x1[:k], x2[:k])
        assert bool((v1[k:] == -7).all())
