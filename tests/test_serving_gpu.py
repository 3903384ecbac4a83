"""Serving: continuous batching of ray chunks of several resident scenes
under CUDA graphs. Each frame's result is the same rendered alone and in a
mix of concurrent requests (bit for bit: the same captured kernels run on
the same chunks), with and without graphs, and close to the synchronising
full-frame served path."""
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
    server = Server(store, chunk_rays=16384, slots=3, max_inflight=4)
    mix = server.run(_requests(), real_time=True)
    alone = []
    for r in _requests():
        r.arrival = 0.0
        alone += server.run([r], real_time=False)
    ext.check_errors(cuda)
    assert any(r.n_chunks > 1 for r in mix)
    for a, b in zip(sorted(mix, key=lambda r: r.rid), sorted(alone, key=lambda r: r.rid)):
        assert torch.equal(a.colors, b.colors), a.rid
        assert torch.equal(a.depths, b.depths), a.rid
        assert a.latency() > 0
    # the same without CUDA graphs
    eager = Server(store, chunk_rays=16384, slots=2, max_inflight=4, use_graph=False)
    for r, a in zip(eager.run(_requests(), real_time=False), sorted(mix, key=lambda r: r.rid)):
        assert torch.equal(r.colors, a.colors)


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
