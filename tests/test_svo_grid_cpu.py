"""The host builder of the leaf-grid octree form (nsvf_svo_grid_build): runs
on the CPU. Grid lines, leaf and flag counts on the workloads' octrees, the
size-then-fill protocol, and the trees it refuses (which then go through the
depth-first kernel)."""
import ctypes

import numpy as np
import pytest

NSVF_OK, NSVF_ERR_OCTREE, NSVF_ERR_CAPACITY = 0, -3, -4


def _build(cen, chi, vs):
    from nsvf_gb300._lib import LIB
    cen = np.ascontiguousarray(cen, np.float32)
    chi = np.ascontiguousarray(chi, np.int32)
    nb = ctypes.c_int64(-1)
    st = LIB.nsvf_svo_grid_build(cen.shape[0], ctypes.c_float(vs), cen.ctypes.data,
                                 chi.ctypes.data, None, 0, ctypes.byref(nb))
    if st != NSVF_ERR_CAPACITY:
        return st, None, None
    blob = np.zeros(nb.value, np.uint8)
    # one byte short is refused, the exact size is filled
    assert LIB.nsvf_svo_grid_build(cen.shape[0], ctypes.c_float(vs), cen.ctypes.data,
                                   chi.ctypes.data, blob.ctypes.data, nb.value - 1,
                                   None) == NSVF_ERR_CAPACITY
    st = LIB.nsvf_svo_grid_build(cen.shape[0], ctypes.c_float(vs), cen.ctypes.data,
                                 chi.ctypes.data, blob.ctypes.data, nb.value, None)
    info = np.zeros(6, np.int32)
    assert LIB.nsvf_svo_grid_info(blob.ctypes.data, info.ctypes.data) == NSVF_OK
    return st, blob, info


@pytest.mark.parametrize("vs,lines,flagged", [(1.0 / 64, (119, 119, 81), False),
                                              (1.0 / 50, (95, 95, 65), True)])
def test_grid_of_shell_octree(vs, lines, flagged):
    from oracle import workload
    p = workload.shell_points(vs)
    cen, chi = workload.octree(p, vs / 2)
    st, blob, info = _build(cen, chi, vs)
    assert st == NSVF_OK
    assert tuple(info[:3]) == lines
    assert info[3] == p.shape[0] and info[5] == cen.shape[0]
    # dyadic voxel sizes: every ancestor's FP32 faces enclose its leaves';
    # at 1/50 some do not, and those leaves carry the ancestor-check flag
    assert (info[4] > 0) == flagged


def _tiny_tree():
    """Root (size 2) with two leaf children at opposite corners."""
    h = 0.5
    cen = np.array([[-h / 2, -h / 2, -h / 2], [h / 2, h / 2, h / 2], [0, 0, 0]], np.float32)
    chi = np.full((3, 9), -1, np.int32)
    chi[0, 8] = chi[1, 8] = 1
    chi[2, :8] = [0, -1, -1, -1, -1, -1, -1, 1]
    chi[2, 8] = 2
    return cen, chi, h


def test_grid_builder_refusals():
    cen, chi, vs = _tiny_tree()
    st, _, info = _build(cen, chi, vs)
    assert st == NSVF_OK and tuple(info[:4]) == (2, 2, 2, 2)
    bad = chi.copy()
    bad[2, 3] = 3                       # a child id >= n
    assert _build(cen, bad, vs)[0] == NSVF_ERR_OCTREE
    bad = chi.copy()
    bad[2, 3] = 0                       # node 0 reached twice
    assert _build(cen, bad, vs)[0] == NSVF_ERR_OCTREE
    c2 = cen.copy()
    c2[1] = c2[0]                       # two leaves in one cell
    assert _build(c2, chi, vs)[0] == NSVF_ERR_OCTREE
    c3 = cen.copy()
    c3[1, 0] += 0.01                    # a centre off the other leaf's grid line... still
    st, _, _ = _build(c3, chi, vs)      # its own line: accepted
    assert st == NSVF_OK
    bad = chi.copy()
    bad[2, 8] = 0                       # a size < 1
    assert _build(cen, bad, vs)[0] == NSVF_ERR_OCTREE
