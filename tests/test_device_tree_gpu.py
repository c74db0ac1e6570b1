"""The tree and interaction lists built on the GPU (hodlr_tree_build_device,
the path hodlr_build takes) equal the reference's on every parity case and
the host restatement's on the edge cases, array for array (HODLRnD
include/HDD_tree.hpp:23-74, include/HDD_clusters.hpp:70-162,
include/HDD_node.hpp:24-31,150-180); a degenerate input is refused with the
same error."""
import os

import numpy as np
import pytest

import cases
from hodlrnd_gb300 import _lib
from hodlrnd_gb300.kernels import Kernel
from hodlrnd_gb300.matrix import HODLRdD_matrix

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
KEYS = ("level_sizes", "node_counts", "nbr_ptr", "nbr", "intr_ptr", "intr", "leaf_perm")


@pytest.mark.parametrize("name", sorted(cases.REF_CASES))
def test_device_tree_matches_reference(name):
    c = cases.REF_CASES[name]
    f = dict(np.load(os.path.join(GOLDEN, f"ref_{name}.npz")))
    M = HODLRdD_matrix(Kernel(c["kind"], c["scale"], c["diag"]), f["points"], *cases.box(c), Nmax=c["nmax"],
                       eps_ACA=c["eps"], INTERACTION_TYPE_ALLOWED=c["dprime"])
    S = M.tree_structure(device=True)
    for k in KEYS:
        assert np.array_equal(S[k], f[k]), k
    assert S["n_far_blocks"] == len(f["blk_rank"])
    M.close()


def _edge_points():
    rng = np.random.default_rng(11)
    yield "clustered_2d", rng.uniform(0, 0.25, (3000, 2)), [0.0, 0.0], [1.0, 1.0], 16, 0
    yield "two_clusters_3d", np.concatenate([rng.uniform(0, 0.2, (2000, 3)), rng.uniform(0.7, 1.0, (2000, 3))]), \
        [0.0] * 3, [1.0] * 3, 32, 0
    yield "one_point", np.array([[0.3, 0.7]]), [0.0, 0.0], [1.0, 1.0], 64, 0
    yield "below_nmax", rng.uniform(-1, 1, (50, 3)), [-1.0] * 3, [1.0] * 3, 64, 0
    yield "line_1d", rng.uniform(0, 1, (4000, 1)), [0.0], [1.0], 32, 0
    yield "five_d", rng.uniform(0, 1, (6000, 5)), [0.0] * 5, [1.0] * 5, 64, -1
    yield "on_split_planes", np.array([[i / 8.0, j / 8.0] for i in range(9) for j in range(9)] * 3), \
        [0.0, 0.0], [1.0, 1.0], 8, 1
    yield "box_not_square", rng.uniform([0, 0, 0], [4, 1, 0.5], (5000, 3)), [0, 0, 0], [4, 1, 0.5], 40, 0
    yield "hodlr3d_n262144", np.random.default_rng(20261203).uniform(0, 1, (262144, 3)), [0.0] * 3, [1.0] * 3, 64, 0


@pytest.mark.parametrize("case", list(_edge_points()), ids=lambda c: c[0])
def test_device_tree_matches_host_tree(case):
    _, pts, lo, hi, nmax, dp = case
    M = HODLRdD_matrix(Kernel("inv_r", 1.0, 1.0), pts, lo, hi, Nmax=nmax, eps_ACA=1e-8, INTERACTION_TYPE_ALLOWED=dp)
    S, H = M.tree_structure(device=True), M.tree_structure()
    for k in KEYS + ("n_far_blocks", "n_near_blocks"):
        assert np.array_equal(S[k], H[k]), k
    M.close()


def test_device_tree_refuses_degenerate_input():
    # 200 copies of one point never split below Nmax = 10 (the reference would
    # loop until it runs out of memory); the device build stops where the host's does
    pts = np.tile([[0.25, 0.25]], (200, 1))
    p = _lib.HodlrParams()
    p.ndim, p.nmax, p.dprime, p.device = 2, 10, 0, 0
    tree = _lib.ctypes.c_void_p()
    D = _lib.ctypes.POINTER(_lib.ctypes.c_double)
    lo, hi = np.zeros(2), np.ones(2)
    rc = _lib.lib().hodlr_tree_build_device(_lib.ctypes.byref(p), np.ascontiguousarray(pts).ctypes.data_as(D), 200,
                                            lo.ctypes.data_as(D), hi.ctypes.data_as(D), _lib.ctypes.byref(tree))
    assert rc == _lib.HODLR_ERR_TREE
    assert "exceeds" in _lib.last_error(None)
