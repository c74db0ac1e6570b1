"""hodlr_aca_block_noalloc: the allocation-free single-block ACA.

Some callers cannot call cudaMalloc where they need a block compressed (their
framework owns all device memory, or they cannot afford cudaMalloc's implicit
synchronisation).  The entry point keeps its bookkeeping in a static device
array and writes only into the caller's buffers.  This test calls it through
the C ABI twice in a row -- a large block (one CTA) then a small one (one warp)
-- and checks each result against the factors that hodlr_build produced for the
same block, within the FP64 parity tolerance of the other GPU tests.  It builds
everything it needs, so it passes alone in a fresh process as well as after the
other tests.  File name chosen so that pytest collects it last.
"""
import ctypes
import os

import numpy as np
import pytest

import cases
from hodlrnd_gb300 import _lib
from hodlrnd_gb300.kernels import Kernel
from hodlrnd_gb300.matrix import HODLRdD_matrix
from oracle.oracle import block_seed

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _bind():
    L = _lib.lib()
    f = L.hodlr_aca_block_noalloc
    P = ctypes.c_void_p
    f.argtypes = [P, ctypes.c_int64, ctypes.c_int32, P, ctypes.c_int32, P, ctypes.c_int32,
                  ctypes.POINTER(_lib.HodlrKernelDesc), ctypes.c_double, ctypes.c_uint64, ctypes.c_int32, P,
                  ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32), P]
    f.restype = ctypes.c_int
    return f


def test_noalloc_block_matches_build():
    torch = pytest.importorskip("torch")
    c = cases.REF_CASES["c1_2d_n2000"]
    f = dict(np.load(os.path.join(GOLDEN, "ref_c1_2d_n2000.npz")))
    pts = f["points"]
    M = HODLRdD_matrix(Kernel(c["kind"], c["scale"], c["diag"]), pts, *cases.box(c), Nmax=c["nmax"],
                       eps_ACA=c["eps"], INTERACTION_TYPE_ALLOWED=c["dprime"])
    M.Assemble_matrix_operators()
    B = M.blocks()
    S = M.tree_structure()
    perm = M.permutation()
    offs = np.concatenate([[0], np.cumsum(S["level_sizes"])])
    begin = np.zeros(offs[-1], np.int64)
    for l in range(len(S["level_sizes"])):
        cnt = S["node_counts"][offs[l]:offs[l + 1]]
        begin[offs[l]:offs[l + 1]] = np.concatenate([[0], np.cumsum(cnt)[:-1]])

    def node(l, k):
        g = offs[l] + k
        return int(begin[g]), int(S["node_counts"][g])

    dims = [max(node(B["level"][b], B["t"][b])[1], node(B["level"][b], B["s"][b])[1]) for b in range(len(B["rank"]))]
    big = next(b for b in range(len(dims)) if dims[b] > 256 and B["rank"][b] < min(dims[b], 512))
    small = next(b for b in range(len(dims)) if dims[b] <= 64 and 0 < B["rank"][b] and not M.block(b)[2])

    d_points = torch.tensor(np.ascontiguousarray(pts.T), dtype=torch.float64, device="cuda")  # ndim x N
    kd = _lib.HodlrKernelDesc(c["kind"], 0, c["scale"], c["diag"])
    fn = _bind()
    stream = torch.cuda.current_stream().cuda_stream
    for b in (big, small):
        l, t, s = int(B["level"][b]), int(B["t"][b]), int(B["s"][b])
        tb, m = node(l, t)
        sb, n = node(l, s)
        # the reference walks a node's points by increasing caller index
        rows = np.sort(perm[tb:tb + m]).astype(np.int32)
        cols = np.sort(perm[sb:sb + n]).astype(np.int32)
        d_rows = torch.tensor(rows, device="cuda")
        d_cols = torch.tensor(cols, device="cuda")
        cap = int(min(m, n, 512))
        d_fac = torch.full(((m + n) * cap,), float("nan"), dtype=torch.float64, device="cuda")
        rank, flags = ctypes.c_int32(-1), ctypes.c_int32(-1)
        rc = fn(d_points.data_ptr(), len(pts), 2, d_rows.data_ptr(), m, d_cols.data_ptr(), n, ctypes.byref(kd),
                c["eps"], block_seed(l, t, s), cap, d_fac.data_ptr(), ctypes.byref(rank), ctypes.byref(flags), stream)
        assert rc == _lib.HODLR_OK, _lib.last_error(None)
        assert flags.value == 0 and rank.value == int(B["rank"][b])
        r = rank.value
        fac = d_fac.cpu().numpy()
        U = fac[:m * cap].reshape(cap, m).T[:, :r]
        V = fac[m * cap:].reshape(cap, n).T[:, :r]
        Ub, Vb, dense = M.block(b)
        assert not dense
        # hodlr_build keeps rows in tree order; put them in the walking order
        Ub = Ub[np.argsort(perm[tb:tb + m], kind="stable")]
        Vb = Vb[np.argsort(perm[sb:sb + n], kind="stable")]
        scale_u = np.abs(Ub).max()
        scale_v = np.abs(Vb).max()
        assert np.abs(U - Ub).max() <= 1e-12 * scale_u
        assert np.abs(V - Vb).max() <= 1e-12 * scale_v
    M.close()


def test_noalloc_rejects_oversized_blocks():
    torch = pytest.importorskip("torch")
    fn = _bind()
    kd = _lib.HodlrKernelDesc(1, 0, 1.0, 1.0)
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    idx = torch.zeros(4, dtype=torch.int32, device="cuda")
    rank, flags = ctypes.c_int32(), ctypes.c_int32()
    too_many = 16384 + 1
    rc = fn(d.data_ptr(), 8, 2, idx.data_ptr(), too_many, idx.data_ptr(), 4, ctypes.byref(kd), 1e-8, 1, 4,
            d.data_ptr(), ctypes.byref(rank), ctypes.byref(flags), 0)
    assert rc == _lib.HODLR_ERR_INVALID and "16384" in _lib.last_error(None)
    rc = fn(d.data_ptr(), 8, 2, idx.data_ptr(), 4, idx.data_ptr(), 4, ctypes.byref(kd), 1e-8, 1, 513,
            d.data_ptr(), ctypes.byref(rank), ctypes.byref(flags), 0)
    assert rc == _lib.HODLR_ERR_INVALID and "512" in _lib.last_error(None)
