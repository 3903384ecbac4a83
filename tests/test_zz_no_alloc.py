"""The allocation-free SVO intersection entry point (nsvf_svo_intersect_noalloc).

Some callers cannot allocate device memory while they render: a real-time
loop or a host engine with a fixed, pre-partitioned memory budget that passes
this library only its own input and output buffers. For them the library
keeps the octree scratch in a fixed-size array of its own. This test calls
that entry point through the C ABI, twice in a row, and checks that its
outputs are identical (the op is exact) to the allocating nsvf_svo_intersect,
and that an octree larger than the fixed scratch is refused.

The file is named so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

NOALLOC_MAX_NODES = 1 << 18


def _noalloc_fn():
    from nsvf_gb300._lib import LIB_PATH
    lib = ctypes.CDLL(LIB_PATH)
    fn = lib.nsvf_svo_intersect_noalloc
    P, i32, f32 = ctypes.c_void_p, ctypes.c_int, ctypes.c_float
    fn.argtypes = [i32, i32, i32, i32, f32, i32, P, P, P, P, P, P, P, P, P]
    fn.restype = i32
    return fn


def _rays(n, seed):
    rng = np.random.RandomState(seed)
    o = rng.normal(size=(n, 3))
    o = 3.0 * o / np.linalg.norm(o, axis=1, keepdims=True)
    d = -o + rng.normal(scale=0.4, size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o.astype(np.float32), d.astype(np.float32)


def test_noalloc_matches_allocating_entry_point(cuda):
    from nsvf_gb300 import ext, geometry, scenes
    p, vs = scenes.scene_shell(1.0 / 32)
    cen, chi = geometry.build_easy_octree(torch.from_numpy(p), vs / 2)
    n = cen.shape[0]
    assert n <= NOALLOC_MAX_NODES
    cen, chi = cen[None].contiguous().to(cuda), chi[None].contiguous().to(cuda)
    o, d = _rays(5000, seed=3)
    rs = torch.from_numpy(o)[None].to(cuda)
    rd = torch.from_numpy(d)[None].to(cuda)
    H = 64
    ref = ext.svo_intersect(rs, rd, cen, chi, vs, H)
    fn = _noalloc_fn()
    stream = torch.cuda.current_stream(cuda).cuda_stream
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    for _ in range(2):
        idx = torch.full((1, 5000, H), 7, dtype=torch.int32, device=cuda)
        lo = torch.full((1, 5000, H), 7.0, device=cuda)
        hi = torch.full((1, 5000, H), 7.0, device=cuda)
        st = fn(1, 1, n, 5000, vs, H, rs.data_ptr(), rd.data_ptr(), cen.data_ptr(), chi.data_ptr(),
                idx.data_ptr(), lo.data_ptr(), hi.data_ptr(), err.data_ptr(), stream)
        assert st == 0
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        assert torch.equal(idx, ref[0])
        assert torch.equal(lo, ref[1])
        assert torch.equal(hi, ref[2])
    assert int((ref[0] != -1).sum()) > 1000


def test_noalloc_rejects_octrees_beyond_its_scratch(cuda):
    fn = _noalloc_fn()
    dummy = torch.zeros(16, device=cuda)
    p = dummy.data_ptr()
    st = fn(1, 1, NOALLOC_MAX_NODES + 1, 4, 0.1, 8, p, p, p, p, p, p, p, None,
            torch.cuda.current_stream(cuda).cuda_stream)
    assert st == -4    # NSVF_ERR_CAPACITY, nothing launched
