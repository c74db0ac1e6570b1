"""BF16 far-field factors (precision "bf16_factors"): U, V and dense far
tiles stored in BF16 with FP32 per-row (dense) and per-column (low-rank)
scales, the near field in FP64, FP64 GMRES.

Tolerances:
* the GPU product of the stored BF16 operator (compensated FP32 sums) equals
  the FP64 product of its dequantised blocks, rebuilt here on the host, to
  1e-10 of |y| -- the scales are applied where the layout says;
* the stored operator differs from the FP64 one by BF16 rounding (2^-9
  relative per entry): at most 3e-3 of |y|;
* a solve at tol 1e-8 on the stored operator converges, and its solution
  leaves a residual of at most 5e-3 against the FP64 operator.
"""
import os

import numpy as np
import pytest

import cases
from hodlrnd_gb300.kernels import Kernel
from hodlrnd_gb300.matrix import HODLRdD_matrix

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def build(c, pts, **kw):
    M = HODLRdD_matrix(Kernel(c["kind"], c["scale"], c["diag"]), pts, *cases.box(c), Nmax=c["nmax"],
                       eps_ACA=c["eps"], INTERACTION_TYPE_ALLOWED=c["dprime"], **kw)
    M.Assemble_matrix_operators()
    return M


def node_rows(M):
    """Per level, the caller indices of each node's points (tree order)."""
    t = M.tree_structure()
    perm = M.permutation()
    out, off = [], 0
    for ls in t["level_sizes"]:
        cnt = t["node_counts"][off:off + ls]
        beg = np.concatenate([[0], np.cumsum(cnt)[:-1]])
        out.append([perm[b:b + c] for b, c in zip(beg, cnt)])
        off += ls
    return out


def dense_of(blk):
    U, V, dense = blk
    return U if dense else U @ V.T


@pytest.mark.parametrize("name", ["hodlr3d_n4096", "hmat2d_log_n3000"])
def test_bf16_product_is_the_stored_operator(name):
    c = cases.REF_CASES[name]
    f = dict(np.load(os.path.join(GOLDEN, f"ref_{name}.npz")))
    M64 = build(c, f["points"])
    Mb = build(c, f["points"], precision="bf16_factors")
    B = M64.blocks()
    assert np.array_equal(Mb.blocks()["rank"], B["rank"])  # same ACA, stored differently
    assert Mb.statistics()["far_bytes"] < 0.5 * M64.statistics()["far_bytes"]
    x = f["x"]
    y64, yb = M64 * x, Mb * x
    rows = node_rows(M64)
    pred = np.zeros_like(y64)
    for b in range(len(B["rank"])):
        lv, t, s = int(B["level"][b]), int(B["t"][b]), int(B["s"][b])
        D = dense_of(Mb.block(b)) - dense_of(M64.block(b))
        pred[rows[lv][t]] += D @ x[rows[lv][s]]
    ny = np.linalg.norm(y64)
    assert np.linalg.norm((yb - y64) - pred) <= 1e-10 * ny
    assert 0 < np.linalg.norm(yb - y64) <= 3e-3 * ny
    M64.close()
    Mb.close()


def test_bf16_solve_backward_error():
    c = cases.REF_CASES["hodlr3d_n4096"]
    f = dict(np.load(os.path.join(GOLDEN, "ref_hodlr3d_n4096.npz")))
    M64 = build(c, f["points"])
    Mb = build(c, f["points"], precision="bf16_factors", max_iter=400)
    x64 = M64.solve(f["b"])
    xb = Mb.solve(f["b"])
    info = Mb.last_solve
    # FP64 iterative refinement around the BF16-operator solves: the residual
    # with the FP64 operator reaches tol, although the stored BF16 operator
    # is about 1e-3 away from it
    assert info["converged"] == 1 and info["rel_residual"] <= c["eps"]
    assert info["outer_iterations"] >= 2
    nb = np.linalg.norm(f["b"])
    assert np.linalg.norm(f["b"] - M64 * xb) <= c["eps"] * nb
    assert np.linalg.norm(xb - x64) <= 1e-5 * np.linalg.norm(x64)
    # without the check: the stored operator's residual, about 1e-3 from the FP64 one
    Mo = build(c, f["points"], precision="bf16_factors", max_iter=400, fp64_check=False)
    xo = Mo.solve(f["b"])
    assert Mo.last_solve["converged"] == 1 and Mo.last_solve["rel_residual"] <= c["eps"]
    assert np.linalg.norm(f["b"] - M64 * xo) <= 5e-3 * nb
    assert Mo.statistics()["device_bytes"] < Mb.statistics()["device_bytes"]
    Mo.close()
    M64.close()
    Mb.close()


def test_bf16_fp32_accumulation():
    """relax="always": every product summed in plain FP32 (FP32 accumulation),
    the true residual included -- within 1e-5 of the compensated products of
    the same stored operator, and a solve at tol 1e-5 converges on it."""
    c = cases.REF_CASES["hodlr3d_n4096"]
    f = dict(np.load(os.path.join(GOLDEN, "ref_hodlr3d_n4096.npz")))
    M64 = build(c, f["points"])
    Mc = build(c, f["points"], precision="bf16_factors")
    Mf = build(c, f["points"], precision="bf16_factors", relax="always", tol=1e-5)
    yc, yf = Mc * f["x"], Mf * f["x"]
    assert not np.array_equal(yc, yf)
    assert np.linalg.norm(yf - yc) <= 1e-5 * np.linalg.norm(yc)
    xf = Mf.solve(f["b"])
    info = Mf.last_solve
    assert info["converged"] == 1 and info["rel_residual"] <= 1e-5
    assert np.linalg.norm(f["b"] - M64 * xf) <= 5e-3 * np.linalg.norm(f["b"])
    for M in (M64, Mc, Mf):
        M.close()
