"""The C-ABI library on the CPU: it loads, exports every symbol the header
declares, validates arguments without touching the GPU, and its host octree
builder matches the golden (reference-built) octree and the oracle."""
import ctypes
import os
import re

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    txt = open(os.path.join(ROOT, "include", "nsvf_gb300.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(nsvf_\w+)\s*\(", txt)))


def test_exports_every_declared_symbol():
    from nsvf_gb300 import _lib
    lib = ctypes.CDLL(_lib.LIB_PATH)
    syms = header_symbols()
    assert len(syms) >= 9
    for s in syms:
        assert hasattr(lib, s), s
    assert set(_lib.exported_symbols()) <= set(syms)


def test_invalid_arguments_are_rejected_on_host():
    from nsvf_gb300._lib import LIB
    assert LIB.nsvf_aabb_intersect(1, 1, 0, 4, 0.1, 8, None, None, None, None, None, None,
                                   None) == -1
    assert LIB.nsvf_svo_intersect(1, 2, 5, 4, 0.1, 8, None, None, None, None, None, None, None,
                                  None, None, None) == -1
    assert LIB.nsvf_status_string(-3) == b"malformed octree"


def test_octree_matches_golden(golden):
    from nsvf_gb300 import geometry
    pts = torch.from_numpy(golden["points"])
    cen, chi = geometry.build_easy_octree(pts, float(golden["voxel_size"]) / 2)
    assert torch.equal(chi, torch.from_numpy(golden["octree_children"]))
    assert torch.equal(cen, torch.from_numpy(golden["octree_centers"]))


def test_octree_matches_oracle_on_shell_scene():
    from nsvf_gb300 import ext, geometry, scenes
    from oracle import cpu
    p, vs = scenes.scene_shell(1.0 / 32)
    coords, _ = geometry.discretize_points(torch.from_numpy(p), vs / 2)
    ranges = coords.max(0)[0] - coords.min(0)[0]
    depth = int(torch.log2(ranges.max().float()).ceil_().long() - 1)
    center = (coords.max(0)[0] + coords.min(0)[0]) / 2
    a = ext.build_octree(center, coords, depth)
    b = cpu.build_octree(center.numpy(), coords.numpy(), depth)
    assert np.array_equal(a[0].numpy(), b[0]) and np.array_equal(a[1].numpy(), b[1])
    # leaves keep their point index, the root is the last row
    assert (a[1][: p.shape[0], 8] == 1).all() and a[1][-1, 8] == 1 << (depth + 1)


def test_octree_rejects_repeated_points():
    from nsvf_gb300 import ext
    from nsvf_gb300._lib import NsvfError
    pts = torch.tensor([[0, 0, 0], [2, 2, 2], [2, 2, 2]])
    with pytest.raises(NsvfError):
        ext.build_octree(torch.tensor([1.0, 1.0, 1.0]), pts, 1)
