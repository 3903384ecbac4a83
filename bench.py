"""Benchmark: full-frame rendering of the 125k-voxel shell scene on GB300.

Workload (the c2 configuration): voxel 1/64 shell of sphere(0.6) U
torus(0.7, 0.2) -> 125,476 voxels, 277,630-node octree; 32-d corner
embeddings N(0, 0.01^2); 4 x 128 ReLU field MLP (Xavier); 800 x 800 pinhole
frames (640,000 rays) from 100 seeded cameras on the radius-4 sphere; SVO
traversal with max_hits 64; inverse-CDF sampling at step voxel/8 = 1/512,
deterministic (eval) jitter; front-to-back compositing; background fill.
A "step" renders one full frame. Synthetic data (seeded), see
nsvf_gb300/scenes.py.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--path plain|served]
    python bench.py --impl reference ...   # the CPU reference arm

Prints one JSON line (rank 0). Timing: CUDA events per frame on the
rendering stream, L2 flushed (256 MB write) between frames outside the timed
events; clocks sampled with nvidia-smi during the timed region.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

RAYS_PER_FRAME = 800 * 800
MAX_HITS = 64
# DRAM bytes per sample of the fused interpolation + MLP kernel, from ncu on a
# 400x400 c2 frame: dram__bytes_read.sum + dram__bytes_write.sum = 125,100,288
# + 46,736,384 bytes for 4,808,670 samples. Most of it is per sample (voxel id
# and position in, sigma and RGB out: 36 B); the 21.9 MB corner table is read
# about once per launch, so scaling by the samples overstates a full frame's
# table reads, while some of the small launch's output writes were still in L2
# when it ended.
MLP_DRAM_BYTES_PER_SAMPLE = (125100288 + 46736384) / 4808670
METRIC = "rays/s (full 800x800 frames)"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--path", default="served", choices=["plain", "served"],
                    help="served: the fused BF16 path (the headline); plain: the drop-in FP32 path")
    ap.add_argument("--plain-steps", type=int, default=3,
                    help="frames of the plain FP32 path timed beside the served path")
    ap.add_argument("--cpu-rays", type=int, default=163840,
                    help="rays of the frame in the CPU baseline sample (about 12 s on one core)")
    ap.add_argument("--ref-rays", type=int, default=0,
                    help="reference arm: seeded rays per frame (0: full 800x800 frames)")
    ap.add_argument("--size", type=int, default=800,
                    help="frame side in pixels (800 = the c2 workload; smaller for profiling)")
    ap.add_argument("--precision", type=int, default=1,
                    help="1: FP8-option frames and max/RMS RGB error vs an FP64 render (c2, and c4 "
                         "with --precision-c4 1)")
    ap.add_argument("--precision-c4", type=int, default=1)
    ap.add_argument("--serve-chunk", type=int, default=262144,
                    help="rays per chunk of the serving pipeline")
    ap.add_argument("--serve-requests", type=int, default=200,
                    help="requests of the multi-scene serving run (c5); 0 skips it")
    return ap.parse_args()


# ---------------------------------------------------------------- workload --

def make_scene(dev, voxel=1.0 / 64):
    import torch
    from nsvf_gb300 import scenes
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.renderer import VolumeRenderer
    p, vs = scenes.scene_shell(voxel)
    args = argparse.Namespace(voxel_size=vs, max_hits=MAX_HITS, raymarching_stepsize_ratio=0.125,
                              voxel_embed_dim=32, use_octree=True, deterministic_step=True,
                              chunk_size=256)
    enc = SparseVoxelEncoder(args, points=p)
    with torch.no_grad():
        enc.values.weight.copy_(scenes.voxel_embeddings(enc.values.weight.shape[0], 32, 0.01, seed=1))
    weights = scenes.stand_in_mlp_weights(seed=2)
    field = StandInField(weights=weights)
    ren = VolumeRenderer(args)
    enc, field, ren = enc.to(dev).eval(), field.to(dev).eval(), ren.eval()
    states = enc.precompute(id=None)
    return dict(points=p, voxel_size=vs, enc=enc, field=field, ren=ren, states=states,
                weights=weights)


def dist_env():
    """(world size, rank, local rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def frame_index(step, rank):
    """Camera of `step` on `rank`: replicas render different frames of the
    same scene (independent work per GPU, weak scaling)."""
    return step + 7 * rank


def max_over_ranks(x, device=None):
    """The largest of a per-rank value over all ranks (a job's time is its
    slowest rank's); x itself when not distributed."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(rays_per_step, steps, world, t_max):
    """Whole-job rays/s: every rank's rays over the slowest rank's time."""
    return rays_per_step * steps * world / t_max


def frame_rays(index, size=800):
    from nsvf_gb300 import scenes
    rs, rd = scenes.frame_view(index % 100, size=size)
    return rs, rd


PRUNE_SIGMA_SCALE = 3.6e5


def precision_bench(dev, sc, size, c4=True, frames=5):
    """The precision workloads: (1) the served frame with E4M3 hidden layers
    (nsvf_field_samples_fp8) timed like the BF16 frame; (2) max/RMS RGB and
    depth error of the served BF16, served FP8 and drop-in FP32 frames
    against a float64 render of the same samples (nsvf_gb300.precision), on
    camera 0 of the c2 scene and, with c4, of the same shell at voxel 1/128."""
    import torch
    from nsvf_gb300 import ext
    from nsvf_gb300.precision import report
    from nsvf_gb300.served import SceneState, render_frame
    out = {}
    scene = SceneState(sc["enc"], sc["field"])
    scene.mlp_fp8()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    cams = [frame_rays(i, size) for i in range(frames + 2)]
    cams = [(torch.from_numpy(r).to(dev), torch.from_numpy(d).to(dev)) for r, d in cams]
    for name, mlp in (("served_bf16", "tc"), ("served_fp8", "tc_fp8")):
        with torch.no_grad():
            for rs, rd in cams[:2]:
                render_frame(scene, rs, rd, mlp=mlp)
            torch.cuda.synchronize()
            ext.KERNEL_TIMING = True
            ext.kernel_events.clear()
            ts = []
            for rs, rd in cams[2:]:
                flush.zero_()
                s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                s0.record()
                render_frame(scene, rs, rd, mlp=mlp)
                e0.record()
                torch.cuda.synchronize()
                ts.append(s0.elapsed_time(e0))
            ext.KERNEL_TIMING = False
            km = ext.kernel_times_ms()
        mk = "field_samples_fp8" if mlp == "tc_fp8" else "field_samples_bf16"
        out[name] = {"rays_per_s": round(size * size * len(ts) / (sum(ts) / 1e3), 1),
                     "ms_per_frame": round(sum(ts) / len(ts), 3),
                     "mlp_ms": round(km[mk]["avg_ms"], 4) if mk in km else None}
    out["frames"] = len(cams) - 2
    workloads = [("c2", sc)]
    if c4:
        workloads.append(("c4", make_scene(dev, 1.0 / 128)))
    for wname, s in workloads:
        rs, rd = cams[0]
        t0 = time.perf_counter()
        rep_ = report(s["enc"], s["field"], s["ren"], rs, rd)
        rep_["voxels"] = int(s["points"].shape[0])
        rep_["seconds"] = round(time.perf_counter() - t0, 1)
        out["errors_vs_fp64_" + wname] = rep_
    return out


def prune_bench(dev, sc, bits=8, th=0.5):
    """The c2 pruning pass: sigma at bits^3 points per voxel, keep voxels with
    max(1 - exp(-relu(sigma) * step)) >= th. Fused BF16 tensor-core kernel
    (nsvf_prune_scores_bf16) vs the FP32 path (offset_points, the FP32
    interpolation kernel, the field's FP32 MLP), with the masks compared."""
    import torch
    from nsvf_gb300 import geometry, scenes
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.functional import trilinear_embed
    from nsvf_gb300.mlp import TensorCoreMLP
    enc, states = sc["enc"], sc["states"]
    # The frame's field is nearly transparent at this step (every alpha far
    # below 0.5, so every voxel would be dropped); the pruning pass uses the
    # same MLP with its density row scaled so that about half of the c2
    # voxels reach the threshold.
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=2, sigma_scale=PRUNE_SIGMA_SCALE)).to(dev).eval()
    centers = states["voxel_center_xyz"].float().contiguous()
    feats = states["voxel_vertex_idx"].int().contiguous()
    values = states["voxel_vertex_emb"].detach().float().contiguous()
    vs, step = float(enc.voxel_size), float(enc.step_size)
    mlp = TensorCoreMLP(field)
    V = centers.shape[0]
    mlp.prune_scores(centers[:256], feats[:256], values, vs, bits=bits, rule=1, step=step)
    torch.cuda.synchronize(dev)
    s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record()
    score = mlp.prune_scores(centers, feats, values, vs, bits=bits, rule=1, step=step)
    e0.record()
    torch.cuda.synchronize(dev)
    keep_bf16 = score >= th
    alpha = torch.empty(V, device=dev)
    hv = torch.tensor(vs / 2.0, device=dev)
    chunk = 8192

    def fp32_pass(stop):
        with torch.no_grad():
            for i in range(0, stop, chunk):
                c = centers[i:i + chunk]
                pts = geometry.offset_points(c, hv, bits=bits).reshape(-1, 3)
                idx = torch.arange(i, i + c.shape[0], device=dev)[:, None].expand(-1, bits ** 3).reshape(-1)
                emb = trilinear_embed(idx, pts, centers, feats, values, vs)
                sig = field.mlp(emb)[:, 0].reshape(-1, bits ** 3)
                alpha[i:i + c.shape[0]] = (1 - torch.exp(-torch.relu(sig) * step)).max(-1)[0]

    # the FP32 path's time varies from run to run (cuBLAS SGEMM on
    # multi-GB activations): one chunk of warm-up, then the faster of two
    # timed passes
    fp32_pass(min(V, chunk))
    torch.cuda.synchronize(dev)
    fp32_ms = []
    for _ in range(2):
        s1, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s1.record()
        fp32_pass(V)
        e1.record()
        torch.cuda.synchronize(dev)
        fp32_ms.append(s1.elapsed_time(e1))
    keep_fp32 = alpha >= th
    # the exact pass: BF16 screen with the error scale M, double-float
    # evaluation of the undecided points (TensorCoreMLP.prune_mask)
    mlp.prune_mask(centers[:256], feats[:256], values, vs, th=th, bits=bits, rule=1, step=step)
    torch.cuda.synchronize(dev)
    ex_ms = []
    for _ in range(2):
        s2, e2 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s2.record()
        keep_exact, _, n_undecided = mlp.prune_mask(centers, feats, values, vs, th=th, bits=bits,
                                                    rule=1, step=step)
        e2.record()
        torch.cuda.synchronize(dev)
        ex_ms.append(s2.elapsed_time(e2))
    return {"workload": "c2 pruning pass: %d voxels x %d^3 points, keep max(1-exp(-relu(s)*step)) >= %g; "
                        "density row of the field scaled by %g" % (V, bits, th, PRUNE_SIGMA_SCALE),
            "exact_ms": round(min(ex_ms), 3),
            "exact_path": "BF16 tensor-core screen (error scale M = sum |W4[0]| h) + double-float "
                          "evaluation of the undecided points; mask of the rule without rounding error",
            "undecided_points": n_undecided, "points": V * bits ** 3,
            "kept_exact": int(keep_exact.sum()),
            "mask_mismatches_exact_vs_fp32": int((keep_exact != keep_fp32).sum()),
            "alpha_fp32_median": float(alpha.median()),
            "bf16_fused_ms": round(s0.elapsed_time(e0), 3), "fp32_ms": round(min(fp32_ms), 3), "fp32_ms_both": [round(t, 1) for t in fp32_ms],
            "tflop": round(107520.0 * V * bits ** 3 / 1e12, 2),
            "bf16_tflops_achieved": round(107520.0 * V * bits ** 3 / (s0.elapsed_time(e0) / 1e3) / 1e12, 1),
            "kept_bf16": int(keep_bf16.sum()), "kept_fp32": int(keep_fp32.sum()),
            "mask_mismatches_bf16_scores_vs_fp32": int((keep_bf16 != keep_fp32).sum()),
            "max_abs_alpha_diff": float((score - alpha).abs().max())}


def train_bench(dev, steps=5, warmup=2):
    """The differentiation workload (c3): the c2 shell, a batch of 4 views
    (cameras 0, 25, 50, 75) x 2,048 pixels drawn among those whose ray hits
    a voxel, targets rendered from a second embedding set, the field's density
    row scaled 30x (bias 0.5). One step = intersection + sampling, the FP32
    forward, the hand-written backward with per-chunk recomputation
    (nsvf_gb300.train), and an Adam step on the embeddings and the field."""
    import torch
    from nsvf_gb300 import ext, scenes, train
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    p, vs = scenes.scene_shell(1.0 / 64)
    args = argparse.Namespace(voxel_size=vs, max_hits=MAX_HITS, raymarching_stepsize_ratio=0.125,
                              voxel_embed_dim=32, use_octree=True, deterministic_step=True)
    enc = SparseVoxelEncoder(args, points=p)
    with torch.no_grad():
        enc.values.weight.copy_(scenes.voxel_embeddings(enc.values.weight.shape[0], 32, 0.01, seed=1))
    field = StandInField(weights=scenes.stand_in_mlp_weights(seed=2, sigma_scale=30.0,
                                                             sigma_bias=0.5))
    enc, field = enc.to(dev), field.to(dev)
    st = enc.precompute(id=None)
    rng = np.random.RandomState(21)
    ro, rd = [], []
    for v in (0, 25, 50, 75):
        rs, rdv = scenes.frame_view(v)
        rdt = torch.from_numpy(rdv).to(dev)
        _, _, _, hits = ext.svo_intersect_sorted(
            torch.from_numpy(rs).to(dev).reshape(1, 1, 3).expand(1, rdt.shape[0], 3).contiguous(),
            rdt[None], st["voxel_octree_center_xyz"].float()[None].contiguous(),
            st["voxel_octree_children_idx"].int()[None].contiguous(), vs, MAX_HITS)
        hit = hits[0].nonzero().squeeze(1).cpu().numpy()
        pix = np.sort(rng.choice(hit, 2048, replace=False))
        ro.append(np.broadcast_to(rs, (2048, 3)))
        rd.append(rdv[pix])
    ro = torch.from_numpy(np.concatenate(ro).astype(np.float32)).to(dev)
    rd = torch.from_numpy(np.concatenate(rd).astype(np.float32)).to(dev)
    with torch.no_grad():
        v0 = enc.values.weight.clone()
        enc.values.weight.copy_(scenes.voxel_embeddings(v0.shape[0], 32, 0.01, seed=7).to(dev))
        target = train.render_batch(enc, field, ro, rd, states=st)
        enc.values.weight.copy_(v0)
    opt = torch.optim.Adam(list(enc.parameters()) + list(field.parameters()), lr=1e-4)
    for _ in range(warmup):
        train.train_step(enc, field, ro, rd, target, optimizer=opt, states=st)
    torch.cuda.synchronize(dev)
    torch.cuda.reset_peak_memory_stats(dev)
    base = torch.cuda.memory_allocated(dev)
    ts, losses = [], []
    for _ in range(steps):
        s0, e0 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s0.record()
        loss = train.train_step(enc, field, ro, rd, target, optimizer=opt, states=st)
        e0.record()
        torch.cuda.synchronize(dev)
        ts.append(s0.elapsed_time(e0))
        losses.append(float(loss))
    smp = train.sample_rays(enc, ro, rd, st)
    return {"workload": "c3: 125,476-voxel shell, 4 views x 2,048 hit pixels, targets from a second "
                        "embedding set, field density x30 (bias 0.5); FP32 forward, hand-written "
                        "backward with per-chunk recomputation (1,024-ray chunks), Adam",
            "ms_per_step": round(statistics.mean(ts), 3), "steps": steps,
            "rays_per_s": round(8192 / (statistics.mean(ts) / 1e3), 1),
            "samples_per_step": int(smp[1].ne(-1).sum()),
            "peak_mem_mb_above_resident": round((torch.cuda.max_memory_allocated(dev) - base) / 2 ** 20, 1),
            "loss_first_last": [round(losses[0], 6), round(losses[-1], 6)]}


def serve_bench(dev, n_requests, rate=200.0, seed=0, chunk_rays=262144, samples_per_ray=128):
    """The c5 serving workload: eight resident seeded scenes (sphere/torus/box
    unions, 10k-400k voxels), each with its own 4x128 MLP; Poisson arrivals at
    `rate`/s, each request one scene at a random camera on the radius-4 sphere
    and a resolution in {128, 256, 512, 800}^2. Served BF16 path (continuous
    batching of 64k-ray chunks on 3 streams, CUDA graphs) vs the plain FP32
    drop-in path rendering a prefix of the same requests one at a time."""
    import torch
    from nsvf_gb300 import scenes
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.renderer import VolumeRenderer, render_rays
    from nsvf_gb300.serving import SceneStore, Server, poisson_requests
    t_setup = time.perf_counter()
    store = SceneStore(dev, 64 << 30)
    plain = {}
    voxels = []
    for sid, (p, vs) in enumerate(scenes.serving_scenes()):
        args = argparse.Namespace(voxel_size=vs, max_hits=MAX_HITS, raymarching_stepsize_ratio=0.125,
                                  voxel_embed_dim=32, use_octree=True, deterministic_step=True,
                                  chunk_size=256)
        enc = SparseVoxelEncoder(args, points=p)
        with torch.no_grad():
            enc.values.weight.copy_(scenes.voxel_embeddings(enc.values.weight.shape[0], 32, 0.01,
                                                            seed=10 + sid))
        field = StandInField(weights=scenes.stand_in_mlp_weights(seed=20 + sid))
        enc, field = enc.to(dev).eval(), field.to(dev).eval()
        store.add(sid, enc, field)
        plain[sid] = (enc, field, VolumeRenderer(args).eval(), enc.precompute(id=None))
        voxels.append(int(p.shape[0]))
    # 256k-ray chunks: fewer, longer launches per frame (64k: 99 M rays/s at
    # capacity, p99 20 ms; 128k: 117 M, 14 ms; 256k: 125 M, 11 ms). A chunk
    # holds up to 128 samples per ray on average (c2 averages 29); one that
    # needs more is rendered again without the cap.
    server = Server(store, chunk_rays=chunk_rays, slots=3, max_inflight=8, frame_budget_bytes=1 << 30,
                    samples_per_ray=samples_per_ray)
    server.warm(list(store.scenes))
    server.reserve_host_buffers(800 * 800, 8)
    reqs = poisson_requests(n_requests, rate, list(store.scenes), [128, 256, 512, 800], seed=seed)
    torch.cuda.synchronize(dev)
    setup_s = time.perf_counter() - t_setup
    t0 = time.perf_counter()
    out = server.run(reqs, real_time=True)
    wall = time.perf_counter() - t0
    lat = np.array([r.latency() for r in out]) * 1e3
    rays = sum(r.rays for r in out)
    # capacity: the same requests all arriving at once (the queue is never
    # empty, so continuous batching runs at its peak rate)
    burst = poisson_requests(n_requests, 1e9, list(store.scenes), [128, 256, 512, 800], seed=seed)
    t0 = time.perf_counter()
    out_b = server.run(burst, real_time=True)
    wall_b = time.perf_counter() - t0
    lat_b = np.array([r.latency() for r in out_b]) * 1e3
    rays_b = sum(r.rays for r in out_b)
    # plain FP32 drop-in path on a prefix of the same requests, one at a time
    n_plain = min(len(reqs), 16)
    t_plain = []
    rays_plain = 0
    for sid, (enc, field, ren, st) in plain.items():      # warm every scene's plain path once
        rs, rd = scenes.pinhole_rays(scenes.sphere_cameras(1, 4.0, 99)[0], 64, 64, 80.0)
        with torch.no_grad():
            render_rays(enc, field, ren, torch.from_numpy(rs).to(dev).reshape(1, 1, 1, 3),
                        torch.from_numpy(rd).to(dev).reshape(1, 1, -1, 3), encoder_states=st)
    torch.cuda.synchronize(dev)
    for r in reqs[:n_plain]:
        enc, field, ren, st = plain[r.scene_id]
        rs, rd = scenes.pinhole_rays(r.cam, r.width, r.height, r.focal)
        rs_t = torch.from_numpy(rs).to(dev).reshape(1, 1, 1, 3)
        rd_t = torch.from_numpy(rd).to(dev).reshape(1, 1, -1, 3)
        torch.cuda.synchronize(dev)
        ts = time.perf_counter()
        with torch.no_grad():
            o = render_rays(enc, field, ren, rs_t, rd_t, encoder_states=st)
        o["colors"].cpu()
        t_plain.append(time.perf_counter() - ts)
        rays_plain += r.rays
    tp = np.array(t_plain) * 1e3
    return {
        "workload": "c5: 8 resident scenes (%d-%d voxels), Poisson %g req/s, resolutions "
                    "{128,256,512,800}^2, %d requests" % (min(voxels), max(voxels), rate, n_requests),
        "served_bf16": {"rays_per_s": round(rays / wall, 1), "p50_ms": round(float(np.percentile(lat, 50)), 2),
                        "p99_ms": round(float(np.percentile(lat, 99)), 2),
                        "offered_rays_per_s": round(rays / reqs[-1].arrival, 1),
                        "wall_s": round(wall, 3), "chunk_rays": chunk_rays, "samples_per_ray_cap": samples_per_ray, "slots": 3,
                        "cuda_graphs": True},
        "served_bf16_capacity": {"rays_per_s": round(rays_b / wall_b, 1),
                                 "p50_ms": round(float(np.percentile(lat_b, 50)), 2),
                                 "p99_ms": round(float(np.percentile(lat_b, 99)), 2),
                                 "note": "all %d requests at t=0; latency includes queueing"
                                         % n_requests},
        "plain_fp32_sequential": {"rays_per_s": round(rays_plain / tp.sum() * 1e3, 1),
                                  "p50_ms": round(float(np.percentile(tp, 50)), 2),
                                  "p99_ms": round(float(np.percentile(tp, 99)), 2),
                                  "requests": n_plain,
                                  "note": "render time per request, no queueing"},
        "setup_s": round(setup_s, 1),
    }


# ------------------------------------------------------------- clocks ------

class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms. start() is
    called before the warm-up and waits for the first sample, so that
    nvidia-smi's own start-up does not overlap the timed frames; mark() and
    stop() bracket the timed region, whose samples (with the one just before
    it) give the reported clocks."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.first = 0

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            t0 = time.time()
            while not self.lines and time.time() - t0 < 10.0 and self.proc.poll() is None:
                time.sleep(0.01)
        except Exception:
            self.proc = None

    def mark(self):
        """The timed region starts: samples from here on (and the last one
        before) are the ones reported."""
        self.first = max(0, len(self.lines) - 1)

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines[self.first:]:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


# ----------------------------------------------------------- GPU arm ---------

def run_ours(a):
    import torch
    import torch.distributed as dist
    from nsvf_gb300 import ext
    from nsvf_gb300._lib import LIB
    from nsvf_gb300.renderer import render_rays

    world, rank, local = dist_env()
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    torch.backends.cuda.matmul.allow_tf32 = False
    torch.backends.cudnn.allow_tf32 = False
    sc = make_scene(dev)
    enc, field, ren, states = sc["enc"], sc["field"], sc["ren"], sc["states"]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # host-resident inputs of every frame (pinned), one camera per step
    n_frames = a.warmup + a.steps
    host = []
    for i in range(n_frames):
        rs, rd = frame_rays(frame_index(i, rank), a.size)
        rdt = torch.from_numpy(rd).pin_memory()
        rst = torch.from_numpy(rs).pin_memory()
        host.append((rst, rdt))
    dev_in = [(h[0].to(dev), h[1].to(dev)) for h in host]

    if a.path == "served":
        from nsvf_gb300.served import SceneState, render_frame
        scene = SceneState(enc, field)

        def step(rs, rd):
            with torch.no_grad():
                return render_frame(scene, rs, rd)
    else:
        def step(rs, rd):
            with torch.no_grad():
                return render_rays(enc, field, ren, rs.reshape(1, 1, 1, 3),
                                   rd.reshape(1, 1, -1, 3), encoder_states=states)

    # --- device-resident timing (value) ---
    clocks = ClockSampler(local)
    clocks.start()
    ext.KERNEL_TIMING = True
    for i in range(a.warmup):
        step(*dev_in[i])
    torch.cuda.synchronize()
    ext.kernel_events.clear()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.mark()
    times = []
    out_samples = [0]
    far_n = [0, 0]
    l0 = LIB.nsvf_launch_count()
    for i in range(a.steps):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        out = step(*dev_in[a.warmup + i])
        e.record()
        torch.cuda.synchronize()
        times.append(s.elapsed_time(e) / 1e3)
        out_samples[0] += int(out.get("n_samples", 0) or 0)
        far_n[0] += int(out.get("n_far_outside", 0) or 0)
        far_n[1] += int(out.get("n_rays_refined_fp32", 0) or 0)
    launches = LIB.nsvf_launch_count() - l0
    clk = clocks.stop()
    ext.KERNEL_TIMING = False
    kernel_ms = ext.kernel_times_ms()
    t_dev = max_over_ranks(sum(times), dev)
    far_stats = {"samples_far_outside_per_frame": far_n[0] / a.steps,
                 "rays_refined_fp32_per_frame": far_n[1] / a.steps,
                 "note": "samples with a trilinear coordinate outside [-0.5, 1.5] (the reference's "
                         "sampling tail) are re-evaluated in double-float; rays where such a "
                         "sample's colour exceeds 1000 get their other samples in FP32"}

    # --- end to end through the public API with host buffers ---
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    e2e_times = []
    h2d = d2h = 0
    # results land in pinned host buffers (as a serving front end would keep)
    col_h = [torch.empty(a.size * a.size, 3, dtype=torch.float32).pin_memory() for _ in range(2)]
    dep_h = [torch.empty(a.size * a.size, dtype=torch.float32).pin_memory() for _ in range(2)]
    h2d = host[a.warmup][0].numel() * 4 + host[a.warmup][1].numel() * 4
    d2h = col_h[0].numel() * 4 + dep_h[0].numel() * 4
    e2e_overlap = a.path == "served"
    if e2e_overlap:
        # served.HostFrames: frame i + 1's rays are copied in and frame i - 1's
        # results copied out while frame i renders; the L2 flush between
        # frames runs inside the timed region, on the rendering stream
        from nsvf_gb300.served import HostFrames
        pipe = HostFrames(scene, a.size * a.size)
        frames = [(host[a.warmup + i][0], host[a.warmup + i][1], col_h[i % 2], dep_h[i % 2])
                  for i in range(a.steps)]
        with torch.no_grad():
            pipe.render(frames[:2])   # allocates the frame buffers
        torch.cuda.synchronize()
        if world > 1:
            dist.barrier()
        t0 = time.perf_counter()
        with torch.no_grad():
            pipe.render(frames, before_frame=lambda i: flush.zero_())
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    else:
        for i in range(a.steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rst, rdt = host[a.warmup + i]
            rs_d = rst.to(dev, non_blocking=True)
            rd_d = rdt.to(dev, non_blocking=True)
            out = step(rs_d, rd_d)
            col_h[0].copy_(out["colors"].reshape(-1, 3), non_blocking=True)
            dep_h[0].copy_(out["depths"].reshape(-1), non_blocking=True)
            torch.cuda.synchronize()
            e2e_times.append(time.perf_counter() - t0)
    t_e2e = max_over_ranks(sum(e2e_times), dev)

    # the plain FP32 kernels on the same cameras, for the BF16-vs-FP32 ratio:
    # (1) the same served chain with the field's FP32 layers (nn.Linear,
    # cuBLAS SGEMM) instead of the tensor-core BF16 kernel -- the ratio's
    # denominator; (2) the drop-in module path (the reference's structure)
    plain_fp32 = plain_dropin = None

    def time_frames(fn, n):
        fn(*dev_in[0])
        pt = []
        for i in range(min(n, a.steps)):
            flush.zero_()
            s_, e_ = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s_.record()
            fn(*dev_in[a.warmup + i])
            e_.record()
            torch.cuda.synchronize()
            pt.append(s_.elapsed_time(e_))
        return {"value": round(a.size * a.size * len(pt) / (sum(pt) / 1e3), 1), "unit": "rays/s",
                "ms_per_step": round(sum(pt) / len(pt), 3), "steps": len(pt)}

    if a.path == "served" and a.plain_steps > 0:
        def chain_fp32(rs, rd):
            with torch.no_grad():
                return render_frame(scene, rs, rd, mlp="fp32")

        def dropin_fp32(rs, rd):
            with torch.no_grad():
                return render_rays(enc, field, ren, rs.reshape(1, 1, 1, 3), rd.reshape(1, 1, -1, 3),
                                   encoder_states=states)
        plain_fp32 = time_frames(chain_fp32, a.plain_steps)
        plain_fp32["path"] = ("served chain (same kernels, same samples) with the field's FP32 layers "
                              "(torch nn.Linear, cuBLAS SGEMM, TF32 off) and the double-float pass")
        plain_dropin = time_frames(dropin_fp32, a.plain_steps)
        plain_dropin["path"] = "drop-in modules (SparseVoxelEncoder / VolumeRenderer), FP32 field"

    if rank != 0:
        dist.destroy_process_group()
        return
    rays_frame = a.size * a.size
    value = job_throughput(rays_frame, a.steps, world, t_dev)
    ms = [x * 1e3 for x in times]
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) \
        if os.path.exists(os.path.join(ROOT, "MEASURED_PEAKS.json")) else None
    hbm_peak = peaks["hbm_gbs"] if peaks else 6800.0
    # roofline of the intersection: the leaf-grid sweep (or the SVO traversal
    # with the fused sort). Algorithmic bytes per launch: R*24 (ray origin +
    # direction) + the octree's form (grid blob, or Nn*48 for the packed
    # octree) + R*H*12 (sorted ids/min/max) + R (hit flags).
    Nn = int(states["voxel_octree_children_idx"].shape[0])
    k = kernel_ms.get("svo_intersect_grid")
    if k:
        g = scene.svo_grid if a.path == "served" else enc._runtime_caches.get("svo_grid")
        tree_bytes = int(g.grid.numel()) if g is not None and g.ok else Nn * 48
        k_name = "svo_intersect_grid (svo_grid_kernel + depth-first list pass)"
    else:
        k = kernel_ms.get("svo_intersect_sorted")
        tree_bytes = Nn * 48
        k_name = "svo_intersect_sorted (pack + svo_kernel<SORTED>)"
    alg = rays_frame * 24 + tree_bytes + rays_frame * MAX_HITS * 12 + rays_frame
    roof = None
    roof_isect = None
    if k:
        ach = alg / (k["avg_ms"] / 1e3) / 1e9
        roof_isect = {"kernel": k_name, "bound": "hbm",
                      "achieved": round(ach, 1), "peak": hbm_peak, "unit": "GB/s",
                      "frac": round(ach / hbm_peak, 4),
                      "peak_source": "measured" if peaks else "fallback",
                      "algorithmic_bytes_per_launch": alg, "avg_launch_ms": round(k["avg_ms"], 4)}
    if a.path == "served" and kernel_ms.get("field_samples_bf16"):
        # the tensor-core MLP dominates the served path: 107,520 FLOP per
        # sample (2 * (32*128 + 3*128*128 + 128*4)) x samples per launch
        km = kernel_ms["field_samples_bf16"]
        flops = 107520.0 * out_samples[0] / max(1, km["launches"]) if out_samples[0] else 0
        ach = flops / (km["avg_ms"] / 1e3) / 1e12
        tpk = peaks["bf16_tflops"] if peaks else 1900.0
        roof = {"kernel": "field_samples_bf16 (mlp_tc_kernel<kSamplesIn>)", "bound": "tensor",
                "achieved": round(ach, 1),
                "peak": tpk, "unit": "TFLOP/s", "frac": round(ach / tpk, 4),
                "peak_source": "measured (bf16 burst)" if peaks else "fallback",
                "algorithmic_flops_per_launch": flops, "avg_launch_ms": km["avg_ms"],
                "traffic": round(MLP_DRAM_BYTES_PER_SAMPLE * out_samples[0] / max(1, km["launches"])),
                "traffic_unit": "bytes per launch",
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one 400x400 launch "
                                  "(4,808,670 samples: 171.8 MB), scaled by the samples per launch"}
    elif k:
        ach = alg / (k["avg_ms"] / 1e3) / 1e9
        roof = {"kernel": k_name, "bound": "hbm", "achieved": round(ach, 1),
                "peak": hbm_peak, "unit": "GB/s", "frac": round(ach / hbm_peak, 4),
                "peak_source": "measured" if peaks else "fallback",
                "algorithmic_bytes_per_launch": alg, "avg_launch_ms": round(k["avg_ms"], 4),
                "traffic": None}
    cpu = cpu_baseline(a.cpu_rays, threads=1)
    serving = serve_bench(dev, a.serve_requests, chunk_rays=a.serve_chunk) \
        if a.serve_requests > 0 and world == 1 else None
    pruning = prune_bench(dev, sc) if world == 1 else None
    training = train_bench(dev) if world == 1 else None
    precision = precision_bench(dev, sc, a.size, c4=bool(a.precision_c4)) \
        if (world == 1 and a.precision and a.path == "served") else None
    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "rays/s", "n_gpus": world,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(statistics.mean(ms), 3),
        "p50_ms": round(float(np.percentile(ms, 50)), 3), "p99_ms": round(float(np.percentile(ms, 99)), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "bf16 MLP / f32 geometry" if a.path == "served" else "f32",
        "data": "synthetic (seeded scene, embeddings, MLP and cameras)",
        "config": {"workload": "c2: 125,476-voxel sphere+torus shell, %dx%d frame, SVO, "
                               "max_hits 64, step 1/512, 4x128 MLP" % (a.size, a.size),
                   "path": a.path,
                   "voxels": int(sc["points"].shape[0]), "octree_nodes": Nn,
                   "samples_per_frame": (out_samples[0] // a.steps) if out_samples[0] else None,
                   "l2": "flushed (256 MB write) between timed frames", "parallelism": "replicas"},
        "e2e": {"value": round(job_throughput(rays_frame, a.steps, world, t_e2e), 1), "unit": "rays/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "copies": ("overlapped with the neighbouring frames' rendering (served.HostFrames); "
                           "L2 flush inside the timed region") if e2e_overlap else "serial"},
        "gpu_launches": int(launches),
        "kernels_ms": kernel_ms,
        "roofline": roof,
        "roofline_intersection": roof_isect,
        "plain_fp32": plain_fp32,
        "speedup_vs_plain_fp32": (round(value / plain_fp32["value"], 2) if plain_fp32 else None),
        "plain_fp32_dropin": plain_dropin,
        "speedup_vs_plain_fp32_dropin": (round(value / plain_dropin["value"], 2) if plain_dropin
                                         else None),
        "far_outside": far_stats,
        "cpu_baseline": cpu,
        "serving": serving,
        "pruning": pruning,
        "training": training,
        "precision": precision,
        "clocks": clk,
    }
    print(json.dumps(line))


# ------------------------------------------------------------ CPU arm --------
# The CPU legs run only the oracle (oracle/: the C restatement of the
# reference's traversal and sampling kernels plus float64 numpy for the
# torch-level parts) on the oracle's own copy of the workload
# (oracle/workload.py): no product module and no product library is loaded.
# Work is spread over spawned worker processes, one ray chunk per task.

_CPU_SCENE = None


def _cpu_worker_init(scene):
    global _CPU_SCENE
    _CPU_SCENE = scene


def _cpu_chunk(args):
    rays_o, rays_d = args
    return cpu_render_chunk(rays_o, rays_d, _CPU_SCENE)


def cpu_render_chunk(rays_o, rays_d, sc):
    """One chunk of rays through the oracle: SVO traversal + depth sort,
    probs/steps (slot-order sum), the reference wrapper's inverse-CDF sampling
    (deterministic jitter), float64 interpolation, MLP and compositing, white
    background. Returns colours [n, 3] and missed [n] (float64)."""
    from oracle import cpu
    vs = sc["voxel_size"]
    cen, chi = sc["octree"]
    step = vs / 8
    n = rays_d.shape[0]
    o = np.broadcast_to(rays_o, (n, 3))[None]
    idx, lo, hi = cpu.sort_hits(*cpu.svo_intersect(o, rays_d[None], cen[None], chi[None], vs,
                                                   MAX_HITS))
    idx, lo, hi = idx[0], lo[0], hi[0]
    hit = (idx != -1).any(-1)
    col = np.zeros((n, 3))
    mis = np.ones(n)
    if hit.sum() > 0:
        I, L, Hh = idx[hit], lo[hit], hi[hit]
        pr, st = cpu.probs_steps(I, L, Hh, step)
        N = I.shape[0]
        M = int(np.ceil(st).max()) + MAX_HITS
        si, sd, ss = cpu.inverse_cdf_op(I, L, Hh, pr, st, np.full((N, M), 0.5, np.float32))
        ss = np.maximum(ss, 0)
        mask = si != -1
        xyz = rays_o[None, None].astype(np.float64) + rays_d[hit][:, None, :] * sd[..., None]
        emb = cpu.trilinear_embed(xyz[mask], si[mask], sc["centers_shifted"], sc["feats"],
                                  sc["values"], vs)
        sig, rgb = cpu.mlp_forward(emb, sc["weights_np"])
        S = np.zeros(mask.shape)
        C = np.zeros(mask.shape + (3,))
        S[mask], C[mask] = sig, rgb
        out = cpu.composite(S, C, sd.astype(np.float64), ss.astype(np.float64), mask)
        col[hit] = out["colors"]
        mis[hit] = out["missed"]
    return col + mis[:, None] * 1.0, mis


class CpuPool:
    """`workers` spawned processes holding the scene (1 = this process).
    BLAS threads are pinned to one per process."""

    def __init__(self, sc, workers):
        self.sc, self.workers, self.ex = sc, workers, None
        if workers > 1:
            import multiprocessing
            from concurrent.futures import ProcessPoolExecutor
            for k in ("OMP_NUM_THREADS", "OPENBLAS_NUM_THREADS", "MKL_NUM_THREADS"):
                os.environ[k] = "1"
            self.ex = ProcessPoolExecutor(max_workers=workers,
                                          mp_context=multiprocessing.get_context("spawn"),
                                          initializer=_cpu_worker_init, initargs=(sc,))
            # start every worker (and its scene copy) before any timing
            list(self.ex.map(_cpu_chunk, [(np.zeros(3, np.float32), np.zeros((1, 3), np.float32)
                                           + np.float32(0.5))] * workers))

    def render(self, rays_o, rays_d, chunk=8192):
        if self.ex is None:
            return cpu_render_chunk(rays_o, rays_d, self.sc)
        parts = [(rays_o, rays_d[i:i + chunk]) for i in range(0, rays_d.shape[0], chunk)]
        res = list(self.ex.map(_cpu_chunk, parts))
        return np.concatenate([r[0] for r in res]), np.concatenate([r[1] for r in res])

    def close(self):
        if self.ex is not None:
            self.ex.shutdown()


def cpu_scene():
    from oracle import workload
    return workload.c2_scene()


def cpu_baseline(n_rays, threads=1):
    """Oracle CPU render of a fixed seeded sample of n_rays rays of frame 0,
    in this process (one core)."""
    from oracle import workload
    sc = cpu_scene()
    rs, rd = workload.frame(0)
    sel = np.random.RandomState(0).choice(rd.shape[0], n_rays, replace=False)
    pool = CpuPool(sc, threads)
    t0 = time.perf_counter()
    pool.render(rs, rd[sel])
    dt = time.perf_counter() - t0
    pool.close()
    return {"value": round(n_rays / dt, 1), "unit": "rays/s", "cores": threads, "kind": "port",
            "sample": "%d seeded rays of the 800x800 frame 0 (oracle C traversal/sampling, "
                      "float64 numpy interpolation/MLP/compositing; oracle workload copy)" % n_rays,
            "seconds": round(dt, 2), "nproc": os.cpu_count()}


def run_reference(a):
    """The CPU reference arm: the oracle port of the reference's path on
    every host core (spawned processes), on full 800x800 frames of the same
    cameras (a.ref_rays > 0 times that many seeded rays per frame instead)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle import workload
    workers = os.cpu_count() or 1
    sc = cpu_scene()
    pool = CpuPool(sc, workers)
    n = a.ref_rays if a.ref_rays > 0 else RAYS_PER_FRAME
    times = []
    for i in range(a.warmup + a.steps):
        rs, rd = workload.frame(i)
        if n < rd.shape[0]:
            rd = rd[np.sort(np.random.RandomState(i).choice(rd.shape[0], n, replace=False))]
        t0 = time.perf_counter()
        pool.render(rs, rd)
        if i >= a.warmup:
            times.append(time.perf_counter() - t0)
    pool.close()
    value = n * len(times) / sum(times)
    full = n == RAYS_PER_FRAME
    line = {"impl": "reference", "metric": METRIC, "value": round(value, 1), "unit": "rays/s",
            "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
            "ms_per_step": round(1e3 * sum(times) / len(times), 2), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded)",
            "config": {"workload": "c2: 125,476-voxel shell, 800x800 frames, SVO, max_hits 64, "
                                   "step 1/512, 4x128 MLP",
                       "rays_per_step": n, "full_frames": full},
            "cpu_baseline": {"value": round(value, 1), "unit": "rays/s", "cores": workers,
                             "kind": "port",
                             "sample": ("full 800x800 frames" if full else
                                        "%d seeded rays per frame" % n) +
                                       ", oracle port (C traversal and sampling, numpy float64 "
                                       "rest), %d worker processes" % workers},
            "e2e": {"value": round(value, 1), "unit": "rays/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)


if __name__ == "__main__":
    main()
