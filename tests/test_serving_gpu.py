"""Serving: continuous batching of ray chunks of several resident scenes
under CUDA graphs, chunks packing pixel ranges (pieces) of several frames of
a scene. Each frame's result is the same rendered alone and in a mix of
concurrent requests -- bit for bit: every piece gets its own launch layout,
so what shares its chunk does not matter -- with and without graphs, under
an HBM budget that forces pipelines to be released, and close to the
synchronising full-frame served path."""
import argparse

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _store(dev):
    from nsvf_gb300 import scenes
    from nsvf_gb300.encoder import SparseVoxelEncoder
    from nsvf_gb300.field import StandInField
    from nsvf_gb300.serving import SceneStore
    store = SceneStore(dev, 8 << 30)
    specs = [(scenes.scene_small(), 20, 60.0), (scenes.scene_shell(1.0 / 24), 64, 30.0),
             (scenes.scene_shell(1.0 / 32), 64, 1.0)]
    for sid, ((p, vs), H, ss) in enumerate(specs):
        args = argparse.Namespace(voxel_size=vs, max_hits=H, raymarching_stepsize_ratio=0.125,
                                  voxel_embed_dim=32, use_octree=True, deterministic_step=True)
        enc = SparseVoxelEncoder(args, points=p)
        with torch.no_grad():
            enc.values.weight.copy_(scenes.voxel_embeddings(enc.values.weight.shape[0], 32, 1.0,
                                                            seed=sid + 1))
        field = StandInField(weights=scenes.stand_in_mlp_weights(seed=sid + 2, sigma_scale=ss,
                                                                 sigma_bias=0.5))
        store.add(sid, enc.to(dev).eval(), field.to(dev).eval())
    return store


def _requests(seed=0):
    from nsvf_gb300.serving import poisson_requests
    return poisson_requests(7, rate=2000.0, scene_ids=[0, 1, 2], resolutions=[64, 128, 200],
                            seed=seed)


def test_same_alone_and_in_the_mix(cuda):
    from nsvf_gb300 import ext
    from nsvf_gb300.serving import Server
    store = _store(cuda)
    server = Server(store, chunk_rays=65536, slots=3, max_inflight=6)
    mix = server.run(_requests(), real_time=False)
    assert server.stats["max_frames_per_chunk"] >= 2      # frames shared chunks
    alone = []
    for r in _requests():
        r.arrival = 0.0
        alone += server.run([r], real_time=False)
    ext.check_errors(cuda)
    assert any(len(r.pieces) > 1 for r in mix)
    for a, b in zip(sorted(mix, key=lambda r: r.rid), sorted(alone, key=lambda r: r.rid)):
        assert torch.equal(a.colors, b.colors), a.rid
        assert torch.equal(a.depths, b.depths), a.rid
        assert a.latency() > 0
    # the same in real time, and without CUDA graphs
    rt = Server(store, chunk_rays=65536, slots=3, max_inflight=4)
    for r, a in zip(sorted(rt.run(_requests(), real_time=True), key=lambda r: r.rid),
                    sorted(mix, key=lambda r: r.rid)):
        assert torch.equal(r.colors, a.colors)
    eager = Server(store, chunk_rays=65536, slots=2, max_inflight=4, use_graph=False)
    for r, a in zip(sorted(eager.run(_requests(), real_time=False), key=lambda r: r.rid),
                    sorted(mix, key=lambda r: r.rid)):
        assert torch.equal(r.colors, a.colors)


def test_hbm_budget_releases_pipelines(cuda):
    """A budget with room for the scenes and one pipeline: slots take turns,
    idle pipelines are released to make room, and the frames are the same as
    with room for all."""
    from nsvf_gb300.serving import ChunkPipeline, Server
    store = _store(cuda)
    big = max(ChunkPipeline.estimate_bytes(sc, 65536, 128) for sc in store.scenes.values())
    tight = Server(store, chunk_rays=65536, slots=3, max_inflight=6,
                   hbm_budget_bytes=store.used + big + (1 << 20))
    roomy = Server(store, chunk_rays=65536, slots=3, max_inflight=6)
    a = sorted(tight.run(_requests(seed=5), real_time=False), key=lambda r: r.rid)
    b = sorted(roomy.run(_requests(seed=5), real_time=False), key=lambda r: r.rid)
    assert tight.stats["pipelines_released"] > 0
    assert tight.device_bytes() <= tight.hbm_budget
    for x, y in zip(a, b):
        assert torch.equal(x.colors, y.colors) and torch.equal(x.depths, y.depths)


def test_served_chunks_match_full_frame(cuda):
    """Chunked serving vs one synchronising full-frame render of the same
    rays: they differ only where the reference's inverse-CDF layout (which
    depends on how many hit rays share a launch) changes a tail sample."""
    from nsvf_gb300.serving import Server, camera_params
    from nsvf_gb300.served import render_frame
    from nsvf_gb300._lib import LIB
    store = _store(cuda)
    server = Server(store, chunk_rays=16384, slots=2)
    for r in server.run(_requests(seed=3), real_time=False):
        sc = store.scenes[r.scene_id]
        cam = torch.from_numpy(camera_params(r.cam, r.width, r.height, r.focal)).to(cuda)
        ro = torch.empty(r.rays, 3, device=cuda)
        rd = torch.empty(r.rays, 3, device=cuda)
        assert LIB.nsvf_pinhole_rays(r.rays, cam.data_ptr(), ro.data_ptr(), rd.data_ptr(),
                                     torch.cuda.current_stream().cuda_stream) == 0
        full = render_frame(sc, ro, rd)
        err = (full["colors"].cpu() - r.colors).abs().max(-1)[0]
        assert float((err > 2e-3).float().mean()) < 5e-3
        assert float(err.mean()) < 1e-4
