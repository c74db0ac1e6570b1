"""GPU parity: the CUDA path through the C ABI against the oracle and the
reference's own results.

Tolerances (FP64 operator):
* tree order, block list: identical to the reference (integer work);
* ACA ranks: identical to the oracle's per-block-generator mode except where
  a norm summed in a different order flips a stopping decision (<= 1% of blocks);
* matvec: within 1e-12 of the oracle where every rank agrees, else within
  eps_ACA; within the reference's own compression error of the dense matvec;
* GMRES: the reference's iteration count +-2, solution within 10 x the larger
  of eps_ACA and the reference's matvec error.
"""
import os

import numpy as np
import pytest

import cases
from hodlrnd_gb300 import _lib
from hodlrnd_gb300.kernels import Kernel, kernel_4d_test
from hodlrnd_gb300.matrix import HODLRdD_matrix
from oracle.oracle import OracleHODLR, dense_matvec

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def build(c, pts, **kw):
    M = HODLRdD_matrix(Kernel(c["kind"], c["scale"], c["diag"]), pts, *cases.box(c), Nmax=c["nmax"],
                       eps_ACA=c["eps"], INTERACTION_TYPE_ALLOWED=c["dprime"], **kw)
    M.Assemble_matrix_operators()
    return M


@pytest.fixture(scope="module", params=sorted(cases.REF_CASES))
def case(request):
    name = request.param
    c = cases.REF_CASES[name]
    f = dict(np.load(os.path.join(GOLDEN, f"ref_{name}.npz")))
    M = build(c, f["points"])
    O = OracleHODLR(f["points"], *cases.box(c), nmax=c["nmax"], dprime=c["dprime"], eps=c["eps"], kind=c["kind"],
                    scale=c["scale"], diag=c["diag"], rng_mode=1)
    yield name, c, f, M, O
    M.close()


def test_tree_order_and_blocks_match_reference(case):
    _, _, f, M, _ = case
    assert np.array_equal(M.permutation(), f["leaf_perm"])
    B = M.blocks()
    assert np.array_equal(B["level"], f["blk_level"])
    assert np.array_equal(B["t"], f["blk_t"])
    assert np.array_equal(B["s"], f["blk_s"])


def test_ranks_match_oracle(case):
    _, _, f, M, O = case
    g = M.blocks()["rank"]
    o = O.blocks()["rank"]
    assert np.mean(g != o) <= 0.01, f"{np.sum(g != o)} of {len(g)} ranks differ"
    st = M.statistics()
    assert st["n_far_blocks"] == len(f["blk_rank"])


def test_matvec_matches_oracle_and_dense(case):
    _, c, f, M, O = case
    y = M * f["x"]
    yo = O.matvec(f["x"])
    same_ranks = np.array_equal(M.blocks()["rank"], O.blocks()["rank"])
    assert rel(y, yo) <= (1e-12 if same_ranks else c["eps"])
    ref_err = float(f["y_dense_rel_err"][0])
    y_dense = dense_matvec(f["points"], f["x"], kind=c["kind"], scale=c["scale"], diag=c["diag"])
    assert rel(y, y_dense) <= 2 * ref_err + c["eps"]
    assert rel(y, f["y"]) <= max(c["eps"], 3 * ref_err)


def test_solve_matches_reference(case):
    _, c, f, M, _ = case
    iters = int(f["gmres_iters"][0])
    if iters >= c["n"]:
        pytest.skip("the reference's GMRES did not converge within max_iter = N on this case")
    x = M.solve(f["b"])
    info = M.last_solve
    assert info["converged"] == 1
    assert abs(info["iterations"] - iters) <= 2
    assert rel(x, f["x_solve"]) <= 10 * max(c["eps"], float(f["y_dense_rel_err"][0]))


def test_multiple_right_hand_sides(case):
    _, _, f, M, _ = case
    rng = np.random.default_rng(3)
    X = rng.standard_normal((M.N, 3))
    Y = M * X
    for k in range(3):
        assert np.array_equal(Y[:, k], M * X[:, k])


def test_golden_pair_kernel4d():
    """The reference's golden vectors data/x_10000.bin, data/rhs_10000.bin
    (kernel_4d_test, numPoints = 10) at its shipped hyper-parameters."""
    g = dict(np.load(os.path.join(GOLDEN, "golden_kernel4d_n10000.npz")))
    k = kernel_4d_test(10)
    c = cases.GOLDEN4D
    M = HODLRdD_matrix(k, k.get_points(), [-1.0] * 4, [1.0] * 4, Nmax=c["nmax"], eps_ACA=c["eps"],
                       INTERACTION_TYPE_ALLOWED=c["dprime"])
    M.Assemble_matrix_operators()
    y = M * g["x"]
    assert rel(y, g["rhs"]) < 20 * c["eps"]
    assert rel(y, g["ref_hodlr"]) < 20 * c["eps"]
    # the reference's own self-check (include/main.cpp:42-57): solve back to x
    x = M.solve(y)
    assert rel(x, g["x"]) < 1e-8
    M.close()


def test_mixed_precision_solve_reaches_tolerance():
    c = cases.REF_CASES["hodlr3d_n4096"]
    f = dict(np.load(os.path.join(GOLDEN, "ref_hodlr3d_n4096.npz")))
    M64 = build(c, f["points"])
    M32 = build(c, f["points"], precision="mixed")
    x64 = M64.solve(f["b"])
    x32 = M32.solve(f["b"])
    info = M32.last_solve
    assert info["converged"] == 1 and info["rel_residual"] <= c["eps"]
    assert info["outer_iterations"] >= 1
    # FP32 factors round each entry to ~6e-8; the two solutions differ by that
    # times the conditioning, far below the compression error
    assert rel(x32, x64) < 1e-5
    # the mixed operator's residual evaluated with the FP64 operator
    r = f["b"] - M64 * x32
    assert np.linalg.norm(r) / np.linalg.norm(f["b"]) < 1e-6
    M64.close()
    M32.close()


def test_fp32_factor_solve_reaches_tolerance():
    """FP32-stored factors, products accumulated in compensated FP32, FP64 GMRES
    (x0 = b, as the reference): converges on the stored operator in about the
    FP64 iteration count, to the same solution within the factor rounding."""
    c = cases.REF_CASES["hodlr3d_n4096"]
    f = dict(np.load(os.path.join(GOLDEN, "ref_hodlr3d_n4096.npz")))
    M64 = build(c, f["points"])
    M32 = build(c, f["points"], precision="fp32_factors")
    y64, y32 = M64 * f["x"], M32 * f["x"]
    assert rel(y32, y64) < 1e-6
    x64 = M64.solve(f["b"])
    it64 = M64.last_solve["iterations"]
    x32 = M32.solve(f["b"])
    info = M32.last_solve
    # the FP64 check: the solve ends on the FP64 operator's residual
    assert info["converged"] == 1 and info["rel_residual"] <= c["eps"]
    assert info["iterations"] <= it64 + 15
    assert rel(x32, x64) < 1e-5
    r = f["b"] - M64 * x32
    assert np.linalg.norm(r) / np.linalg.norm(f["b"]) <= c["eps"]
    M64.close()
    M32.close()


def _oracle_compare(pts, lo, hi, nmax, dp, eps, kind, scale, diag):
    O = OracleHODLR(pts, lo, hi, nmax=nmax, dprime=dp, eps=eps, kind=kind, scale=scale, diag=diag, rng_mode=1)
    M = HODLRdD_matrix(Kernel(kind, scale, diag), pts, lo, hi, Nmax=nmax, eps_ACA=eps, INTERACTION_TYPE_ALLOWED=dp)
    M.Assemble_matrix_operators()
    x = np.random.default_rng(5).uniform(-1, 1, len(pts))
    y, yo = M * x, O.matvec(x)
    M.close()
    return y, yo


@pytest.mark.parametrize("name", ["one_point", "below_nmax", "clustered_2d", "line_1d", "split_planes"])
def test_edge_cases_match_oracle(name):
    rng = np.random.default_rng(9)
    if name == "one_point":
        args = (np.array([[0.5, 0.5]]), [0.0, 0.0], [1.0, 1.0], 64, 0)
    elif name == "below_nmax":
        args = (rng.uniform(-1, 1, (50, 3)), [-1.0] * 3, [1.0] * 3, 64, 0)
    elif name == "clustered_2d":  # many empty leaves with non-empty far partners
        args = (rng.uniform(0, 0.25, (3000, 2)), [0.0, 0.0], [1.0, 1.0], 16, 0)
    elif name == "line_1d":
        args = (rng.uniform(0, 1, (4000, 1)), [0.0], [1.0], 32, 0)
    else:  # points exactly on split planes go to the upper child (HDD_clusters.hpp:124-127)
        args = (np.array([[i / 8.0, j / 8.0] for i in range(9) for j in range(9)] * 2) + 1e-3 * np.repeat(
            np.arange(2), 81)[:, None], [0.0, 0.0], [1.0, 1.0], 8, 1)
    pts, lo, hi, nmax, dp = args
    y, yo = _oracle_compare(pts, lo, hi, nmax, dp, 1e-8, 1, 1.0 / len(pts), 1.0)
    assert rel(y, yo) <= 1e-8


def test_device_pointer_entry_points():
    torch = pytest.importorskip("torch")
    c = cases.REF_CASES["c1_2d_n2000"]
    f = dict(np.load(os.path.join(GOLDEN, "ref_c1_2d_n2000.npz")))
    M = build(c, f["points"])
    x = torch.tensor(f["x"], dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    stream = torch.cuda.current_stream().cuda_stream
    M.matvec_device(x.data_ptr(), y.data_ptr(), 1, stream)
    torch.cuda.synchronize()
    assert np.array_equal(y.cpu().numpy(), M * f["x"])
    b = torch.tensor(f["b"], dtype=torch.float64, device="cuda")
    xs = torch.empty_like(b)
    info = M.solve_device(b.data_ptr(), xs.data_ptr(), 1, stream)
    torch.cuda.synchronize()
    assert info["converged"] == 1
    assert rel(xs.cpu().numpy(), M.solve(f["b"])) < 1e-14
    M.close()


def test_budget_is_enforced():
    c = cases.REF_CASES["c1_2d_n2000"]
    f = dict(np.load(os.path.join(GOLDEN, "ref_c1_2d_n2000.npz")))
    with pytest.raises(_lib.HodlrError) as e:
        build(c, f["points"], device_budget_bytes=1 << 16)
    assert e.value.code == _lib.HODLR_ERR_BUDGET


def test_cgs2_orthogonalisation_matches_mgs():
    """CGS2 (six launches per Arnoldi step) against the reference's MGS on the
    FP64 operator: same iteration count within 2, same solution within 1e-10."""
    c = cases.REF_CASES["hodlr3d_n4096"]
    f = dict(np.load(os.path.join(GOLDEN, "ref_hodlr3d_n4096.npz")))
    Mm = build(c, f["points"], ortho="mgs")
    Mc = build(c, f["points"], ortho="cgs2")
    xm = Mm.solve(f["b"])
    xc = Mc.solve(f["b"])
    im, ic = Mm.last_solve, Mc.last_solve
    assert ic["converged"] == 1 and ic["rel_residual"] <= c["eps"]
    assert abs(im["iterations"] - ic["iterations"]) <= 2
    assert rel(xc, xm) < 1e-10
    Mm.close()
    Mc.close()


def test_relaxed_products_keep_the_true_residual():
    """FP32 factors: plain-FP32 products once the residual estimate allows it
    (inexact GMRES); the true residual decides -- with the FP64 operator
    (the FP64 check), or without the check with compensated products on the
    stored operator."""
    c = cases.REF_CASES["hodlr3d_n4096"]
    f = dict(np.load(os.path.join(GOLDEN, "ref_hodlr3d_n4096.npz")))
    M64 = build(c, f["points"])
    Mr = build(c, f["points"], precision="fp32_factors")
    Mc = build(c, f["points"], precision="fp32_factors", relax=False)
    Ms = build(c, f["points"], precision="fp32_factors", fp64_check=False)
    xr, xc, xs = Mr.solve(f["b"]), Mc.solve(f["b"]), Ms.solve(f["b"])
    ir, ic, is_ = Mr.last_solve, Mc.last_solve, Ms.last_solve
    nb = np.linalg.norm(f["b"])
    for x, info in ((xr, ir), (xc, ic)):
        assert info["converged"] == 1 and info["rel_residual"] <= c["eps"]
        # the FP64 operator's residual, recomputed here
        assert np.linalg.norm(f["b"] - M64 * x) <= c["eps"] * nb
    assert rel(xr, xc) < 1e-6
    # no check: the stored operator's true residual, with compensated products
    assert is_["converged"] == 1 and is_["rel_residual"] <= c["eps"]
    assert np.linalg.norm(f["b"] - Mc * xs) <= c["eps"] * nb
    for M in (M64, Mr, Mc, Ms):
        M.close()


@pytest.mark.parametrize("precision", ["fp64", "fp32_factors", "mixed", "bf16_factors"])
def test_operator_file_round_trip(tmp_path, precision):
    """hodlr_op_save / hodlr_op_load: the loaded operator (tree and near field
    rebuilt, far field from the file, no ACA) gives the same bits."""
    c = cases.REF_CASES["hodlr3d_n4096"]
    f = dict(np.load(os.path.join(GOLDEN, "ref_hodlr3d_n4096.npz")))
    M = build(c, f["points"], precision=precision)
    path = tmp_path / "op.bin"
    M.save(path)
    L = HODLRdD_matrix.load(path)
    assert L.statistics()["n_far_blocks"] == M.statistics()["n_far_blocks"]
    assert L.statistics()["far_bytes"] == M.statistics()["far_bytes"]
    assert np.array_equal(L.blocks()["rank"], M.blocks()["rank"])
    assert np.array_equal(L * f["x"], M * f["x"])
    assert np.array_equal(L.solve(f["b"]), M.solve(f["b"]))
    # a damaged file is refused
    blob = path.read_bytes()
    (tmp_path / "cut.bin").write_bytes(blob[:len(blob) // 2])
    with pytest.raises(_lib.HodlrError) as e:
        HODLRdD_matrix.load(tmp_path / "cut.bin")
    assert e.value.code == _lib.HODLR_ERR_IO
    L.close()
    M.close()
