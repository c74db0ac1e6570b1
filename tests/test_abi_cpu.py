"""C ABI checks that need no GPU: the library loads, exports every entry point
declared in include/hodlrnd.h, validates its arguments, and its host-side
tree / interaction lists equal the reference's (HODLRnD include/HDD_tree.hpp:23-74,
include/HDD_node.hpp:150-180) on every parity case and on edge cases."""
import ctypes
import os
import re

import numpy as np
import pytest

import cases
from hodlrnd_gb300 import _lib
from hodlrnd_gb300.matrix import HODLRdD_matrix
from hodlrnd_gb300.kernels import Kernel
from oracle.oracle import OracleHODLR

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module", autouse=True)
def built_library():
    if not os.path.exists(_lib.LIB_PATH):
        from hodlrnd_gb300 import build
        build.build()


def declared_symbols():
    syms = set()
    for name in os.listdir(os.path.join(ROOT, "include")):
        if name.endswith(".h"):
            text = open(os.path.join(ROOT, "include", name)).read()
            syms |= set(re.findall(r"^\s*(?:int|void|uint64_t|const char\s*\*)\s+(hodlr_\w+)\s*\(", text, re.M))
    return sorted(syms)


def test_exports_every_declared_symbol():
    syms = declared_symbols()
    assert len(syms) >= 17
    L = _lib.lib()
    for s in syms:
        assert hasattr(L, s), s


def test_params_default_are_the_reference_defaults():
    p = _lib.HodlrParams()
    _lib.lib().hodlr_params_default(ctypes.byref(p))
    assert (p.ndim, p.nmax, p.dprime, p.restart, p.eps_aca, p.precision) == (2, 64, 0, 100, 1e-10, 0)


@pytest.mark.parametrize("field,value", [("ndim", 0), ("ndim", 9), ("dprime", 2), ("dprime", -2), ("nmax", 0),
                                         ("eps_aca", 0.0), ("eps_aca", 2.0), ("precision", 7), ("relax", 3),
                                         ("ortho", 5)])
def test_ctx_create_rejects_bad_parameters(field, value):
    L = _lib.lib()
    p = _lib.HodlrParams()
    L.hodlr_params_default(ctypes.byref(p))
    setattr(p, field, value)
    ctx = ctypes.c_void_p()
    rc = L.hodlr_ctx_create(ctypes.byref(p), ctypes.byref(ctx))
    assert rc == _lib.HODLR_ERR_INVALID
    assert not ctx
    assert _lib.last_error(None)


def test_relax_codes():
    assert _lib.relax_code(True) == _lib.HODLR_RELAX_AUTO
    assert _lib.relax_code(False) == _lib.HODLR_RELAX_OFF
    assert _lib.relax_code("always") == _lib.HODLR_RELAX_ALWAYS
    with pytest.raises(ValueError):
        _lib.relax_code("sometimes")


def test_null_arguments_are_rejected():
    L = _lib.lib()
    assert L.hodlr_ctx_create(None, None) == _lib.HODLR_ERR_INVALID
    assert L.hodlr_build(None, None, 0, None, None, None, None) == _lib.HODLR_ERR_INVALID
    assert L.hodlr_matvec(None, None, None, 1) == _lib.HODLR_ERR_INVALID
    assert L.hodlr_solve(None, None, None, 1, None) == _lib.HODLR_ERR_INVALID
    assert L.hodlr_op_destroy(None) == _lib.HODLR_OK
    assert L.hodlr_ctx_destroy(None) == _lib.HODLR_OK


@pytest.mark.parametrize("name", sorted(cases.REF_CASES))
def test_host_tree_matches_reference(name):
    c = cases.REF_CASES[name]
    f = dict(np.load(os.path.join(GOLDEN, f"ref_{name}.npz")))
    M = HODLRdD_matrix(Kernel(c["kind"], c["scale"], c["diag"]), f["points"], *cases.box(c), Nmax=c["nmax"],
                       eps_ACA=c["eps"], INTERACTION_TYPE_ALLOWED=c["dprime"])
    S = M.tree_structure()
    for k in ("level_sizes", "node_counts", "nbr_ptr", "nbr", "intr_ptr", "intr", "leaf_perm"):
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


@pytest.mark.parametrize("case", list(_edge_points()), ids=lambda c: c[0])
def test_host_tree_matches_oracle_on_edge_cases(case):
    _, pts, lo, hi, nmax, dp = case
    O = OracleHODLR(pts, lo, hi, nmax=nmax, dprime=dp, eps=1e-8, kind=1, scale=1.0, diag=1.0, with_operators=False)
    ref = O.structure()
    M = HODLRdD_matrix(Kernel("inv_r", 1.0, 1.0), pts, lo, hi, Nmax=nmax, eps_ACA=1e-8, INTERACTION_TYPE_ALLOWED=dp)
    S = M.tree_structure()
    for k in ("level_sizes", "node_counts", "nbr_ptr", "nbr", "intr_ptr", "intr", "leaf_perm"):
        assert np.array_equal(S[k], ref[k]), k
    M.close()


def test_degenerate_tree_is_refused():
    # 200 copies of one point can never be split below Nmax = 10: the
    # reference would loop until it runs out of memory.
    pts = np.tile([[0.25, 0.25]], (200, 1))
    with pytest.raises(_lib.HodlrError) as e:
        HODLRdD_matrix(Kernel("inv_r"), pts, [0, 0], [1, 1], Nmax=10)
    assert e.value.code == _lib.HODLR_ERR_TREE
