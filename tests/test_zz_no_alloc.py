"""The allocation-free SVO intersection entry point (nsvf_svo_intersect_noalloc).

Some callers cannot allocate device memory while they render: a real-time
loop or a host engine with a fixed, pre-partitioned memory budget that passes
this library only its own input and output buffers. For them the library
keeps the octree scratch in a fixed-size array of its own. This test calls
that entry point through the C ABI, twice in a row, and checks that its
outputs are identical (the op is exact) to the allocating nsvf_svo_intersect
and that the repeat call takes no device memory; that octrees beyond the
fixed scratch are refused; and that it works filled to its capacity.

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
    outs = [(torch.full((1, 5000, H), 7, dtype=torch.int32, device=cuda),
             torch.full((1, 5000, H), 7.0, device=cuda), torch.full((1, 5000, H), 7.0, device=cuda))
            for _ in range(2)]
    free = []
    for idx, lo, hi in outs:
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info(cuda)[0])
        st = fn(1, 1, n, 5000, vs, H, rs.data_ptr(), rd.data_ptr(), cen.data_ptr(), chi.data_ptr(),
                idx.data_ptr(), lo.data_ptr(), hi.data_ptr(), err.data_ptr(), stream)
        assert st == 0
        torch.cuda.synchronize()
        assert int(err.item()) == 0
        assert torch.equal(idx, ref[0])
        assert torch.equal(lo, ref[1])
        assert torch.equal(hi, ref[2])
    # the second call took no device memory (the first may have set up the
    # context's module); outputs were allocated before either call
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(cuda)[0] == free[1]
    assert int((ref[0] != -1).sum()) > 1000


def test_noalloc_rejects_octrees_beyond_its_scratch(cuda):
    """More than NSVF_NOALLOC_MAX_NODES nodes in all -- one large octree, or
    b_pts point sets whose product of counts exceeds it -- is refused before
    anything is launched."""
    fn = _noalloc_fn()
    dummy = torch.zeros(16, device=cuda)
    p = dummy.data_ptr()
    s = torch.cuda.current_stream(cuda).cuda_stream
    assert fn(1, 1, NOALLOC_MAX_NODES + 1, 4, 0.1, 8, p, p, p, p, p, p, p, None, s) == -4
    half = NOALLOC_MAX_NODES // 2 + 1
    assert fn(2, 2, half, 4, 0.1, 8, p, p, p, p, p, p, p, None, s) == -4


def test_noalloc_at_its_capacity(cuda):
    """b_pts copies of a small octree filling the scratch to within one copy
    of NSVF_NOALLOC_MAX_NODES (176 bytes per node, the root boxes included),
    one ray per copy: the same outputs as the allocating entry point."""
    from nsvf_gb300 import ext, geometry, scenes
    p, vs = scenes.scene_small()
    cen, chi = geometry.build_easy_octree(torch.from_numpy(p), vs / 2)
    n = cen.shape[0]
    b = NOALLOC_MAX_NODES // n
    assert b * n > NOALLOC_MAX_NODES - n
    cen_b = cen[None].expand(b, n, 3).contiguous().to(cuda)
    chi_b = chi[None].expand(b, n, 9).contiguous().to(cuda)
    o, d = _rays(b, seed=5)
    rs = torch.from_numpy(o).reshape(b, 1, 3).to(cuda)
    rd = torch.from_numpy(d).reshape(b, 1, 3).to(cuda)
    H = 20
    ref = ext.svo_intersect(rs, rd, cen_b, chi_b, vs, H)
    idx = torch.empty(b, 1, H, dtype=torch.int32, device=cuda)
    lo, hi = torch.empty(b, 1, H, device=cuda), torch.empty(b, 1, H, device=cuda)
    err = torch.zeros(1, dtype=torch.int32, device=cuda)
    fn = _noalloc_fn()
    st = fn(b, b, n, 1, vs, H, rs.data_ptr(), rd.data_ptr(), cen_b.data_ptr(), chi_b.data_ptr(),
            idx.data_ptr(), lo.data_ptr(), hi.data_ptr(), err.data_ptr(),
            torch.cuda.current_stream(cuda).cuda_stream)
    assert st == 0
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    assert torch.equal(idx, ref[0]) and torch.equal(lo, ref[1]) and torch.equal(hi, ref[2])
    assert int((ref[0] != -1).sum()) > 100
