"""The oracle's copy of the c2 workload (oracle/workload.py, used by the CPU
legs of bench.py so that they load no product code) equals the product's
workload bit for bit: voxel centres, octree, corner table, embeddings, field
weights and camera rays. Runs on the CPU (the product's host octree builder
needs no GPU)."""
import numpy as np
import pytest
import torch


@pytest.mark.parametrize("vs,n", [(1.0 / 64, 125476), (1.0 / 128, 500832)])
def test_oracle_workload_equals_product_workload(vs, n):
    from nsvf_gb300 import geometry, scenes
    from oracle import workload
    sc = workload.c2_scene(vs)
    p, _ = scenes.scene_shell(vs)
    assert np.array_equal(sc["points"], p) and p.shape[0] == n
    cen, chi = geometry.build_easy_octree(torch.from_numpy(p), vs / 2)
    assert np.array_equal(sc["octree"][0], cen.numpy())
    assert np.array_equal(sc["octree"][1], chi.numpy())
    _, feats = geometry.voxel_corner_table(torch.from_numpy(p), vs)
    assert np.array_equal(sc["feats"], feats.numpy())
    assert np.array_equal(sc["values"], scenes.voxel_embeddings(feats.max().item() + 1, 32, 0.01,
                                                                seed=1).numpy())
    for (W, b), (W2, b2) in zip(sc["weights_np"], scenes.stand_in_mlp_weights(seed=2)):
        assert np.array_equal(W, W2.numpy()) and np.array_equal(b, b2.numpy())
    for i in (0, 7, 123):
        rs, rd = workload.frame(i)
        rs2, rd2 = scenes.frame_view(i % 100)
        assert np.array_equal(rs, rs2) and np.array_equal(rd, rd2)
