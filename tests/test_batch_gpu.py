"""Batches (hodlr_build_batch): every instance's blocks compressed in shared
ACA launches get the ranks an operator built alone gets (same per-block
generator seeds, same arithmetic, the instance's own kernel scale); the
merged-plan matvec, captured as a CUDA graph, gives bit for bit what each
operator's own matvec gives, on the first (captured) call and on replays."""
import ctypes

import numpy as np
import pytest

from hodlrnd_gb300 import _lib
from hodlrnd_gb300.batch import HODLRdD_batch
from hodlrnd_gb300.kernels import Kernel
from hodlrnd_gb300.matrix import HODLRdD_matrix

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def instances(count=5, seed=23):
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        n = int(rng.integers(1500, 6000))
        pts = rng.uniform(0.0, 1.0, (n, 3))
        out.append((pts, Kernel("inv_r", 1.0 / n ** (2.0 / 3.0), 1.0)))
    return out


def ranks_of(op, nb):
    lv, t, s = np.zeros(nb, np.int32), np.zeros(nb, np.int64), np.zeros(nb, np.int64)
    r = np.zeros(nb, np.int32)
    I32, I64 = ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int64)
    _lib.check(_lib.lib().hodlr_get_blocks(op, lv.ctypes.data_as(I32), t.ctypes.data_as(I64), s.ctypes.data_as(I64),
                                           r.ctypes.data_as(I32)))
    return r


@pytest.mark.parametrize("precision", ["fp64", "fp32_factors"])
def test_batch_matches_operators_built_alone(precision):
    inst = instances()
    box = ([0.0] * 3, [1.0] * 3)
    params = dict(Nmax=64, eps_ACA=1e-6, precision=precision)
    B = HODLRdD_batch([k for _, k in inst], [p for p, _ in inst], [box] * len(inst), **params)
    alone = [HODLRdD_matrix(k, p, *box, **params).Assemble_matrix_operators() for p, k in inst]
    for i, M in enumerate(alone):
        nb = M.statistics()["n_far_blocks"]
        assert np.array_equal(ranks_of(B.op(i), nb), M.blocks()["rank"])
    off = B.offsets
    nrhs = 3
    rng = np.random.default_rng(1)
    X = torch.tensor(rng.standard_normal((nrhs, off[-1])), dtype=torch.float64, device="cuda")
    Y = torch.empty_like(X)
    st = torch.cuda.current_stream().cuda_stream
    B.matvec_device(X.data_ptr(), Y.data_ptr(), nrhs, st)  # captured, then launched
    torch.cuda.synchronize()
    Y1 = Y.cpu().numpy().copy()
    Y.zero_()
    B.matvec_device(X.data_ptr(), Y.data_ptr(), nrhs, st)  # replayed
    torch.cuda.synchronize()
    assert np.array_equal(Y.cpu().numpy(), Y1)
    for i, M in enumerate(alone):
        for c in range(nrhs):
            xi = X[c, off[i]:off[i + 1]].contiguous()
            yi = torch.empty_like(xi)
            M.matvec_device(xi.data_ptr(), yi.data_ptr(), 1, st)
            torch.cuda.synchronize()
            assert np.array_equal(Y1[c, off[i]:off[i + 1]], yi.cpu().numpy())
        M.close()
    B.close()


def test_mixed_batch_fp32_vectors_and_solves():
    inst = instances(4, seed=5)
    box = ([0.0] * 3, [1.0] * 3)
    params = dict(Nmax=64, eps_ACA=1e-6, precision="mixed", tol=1e-6)
    B = HODLRdD_batch([k for _, k in inst], [p for p, _ in inst], [box] * len(inst), **params)
    off = B.offsets
    rng = np.random.default_rng(2)
    # 40 right-hand sides: two chunks of 32 (the second padded) of the
    # multi-RHS kernels, each factor byte read once per chunk
    nrhs = 40
    X = torch.tensor(rng.standard_normal((nrhs, off[-1])), dtype=torch.float32, device="cuda")
    Y = torch.empty_like(X)
    B.matvec_device(X.data_ptr(), Y.data_ptr(), nrhs, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    for i, (p, k) in enumerate(inst):
        M = HODLRdD_matrix(k, p, *box, Nmax=64, eps_ACA=1e-6).Assemble_matrix_operators()
        for c in (0, 1, 31, 32, 39):
            x = X[c, off[i]:off[i + 1]].double().cpu().numpy()
            y = M * x
            assert np.linalg.norm(Y[c, off[i]:off[i + 1]].double().cpu().numpy() - y) / np.linalg.norm(y) < 1e-5
        # the instance is an ordinary operator for solves
        b = rng.standard_normal(p.shape[0])
        x = np.zeros_like(b)
        info = _lib.HodlrSolveInfo()
        D = ctypes.POINTER(ctypes.c_double)
        _lib.check(_lib.lib().hodlr_solve(B.op(i), b.ctypes.data_as(D), x.ctypes.data_as(D), 1, ctypes.byref(info)))
        assert info.converged == 1
        assert np.linalg.norm(b - M * x) / np.linalg.norm(b) < 1e-5
        M.close()
    B.close()
