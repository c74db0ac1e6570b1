"""Test-oracle only: ctypes binding of the CPU restatement (hodlr_oracle.cpp).

Used by tests/ as the checker and by bench.py's CPU-baseline leg; the GPU
product never imports it.
"""
import ctypes
import os

import numpy as np

from . import build as _build

KERNEL_INV_R, KERNEL_INV_R2, KERNEL_LOG_R, KERNEL_EXP_NEG_R = 1, 2, 3, 4


class _Params(ctypes.Structure):
    _fields_ = [("ndim", ctypes.c_int32), ("nmax", ctypes.c_int32), ("dprime", ctypes.c_int32),
                ("kind", ctypes.c_int32), ("eps", ctypes.c_double), ("scale", ctypes.c_double),
                ("diag", ctypes.c_double), ("rng_mode", ctypes.c_int32), ("threads", ctypes.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "liboracle.so")
        if not os.path.exists(path):
            _build.build_oracle()
        L = ctypes.CDLL(path)
        P, D, I64 = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int64)
        L.orc_build.restype = P
        L.orc_build.argtypes = [ctypes.POINTER(_Params), D, ctypes.c_int64, D, D, ctypes.c_int32]
        L.orc_free.argtypes = [P]
        L.orc_num_levels.restype = ctypes.c_int64
        L.orc_num_levels.argtypes = [P]
        L.orc_level_size.restype = ctypes.c_int64
        L.orc_level_size.argtypes = [P, ctypes.c_int64]
        L.orc_structure_sizes.argtypes = [P, I64]
        L.orc_get_structure.argtypes = [P, I64, I64, I64, I64, I64, I64]
        L.orc_num_blocks.restype = ctypes.c_int64
        L.orc_num_blocks.argtypes = [P]
        L.orc_get_blocks.argtypes = [P, I64, I64, I64, I64, I64]
        L.orc_get_block_factors.argtypes = [P, ctypes.c_int64, D, D]
        L.orc_matvec.argtypes = [P, D, D]
        L.orc_gmres.restype = ctypes.c_int32
        L.orc_gmres.argtypes = [P, D, D, ctypes.c_int32, ctypes.c_int32, ctypes.c_double, D]
        L.orc_stats.argtypes = [P, D]
        L.orc_dense_matvec.argtypes = [ctypes.POINTER(_Params), D, ctypes.c_int64, D, I64, ctypes.c_int64, D]
        L.orc_dense_gmres.restype = ctypes.c_int32
        L.orc_dense_gmres.argtypes = [ctypes.POINTER(_Params), D, ctypes.c_int64, D, D, ctypes.c_int32,
                                      ctypes.c_int32, ctypes.c_double, D]
        L.orc_block_seed.restype = ctypes.c_uint64
        L.orc_block_seed.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _q(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))


def make_params(ndim, nmax, dprime, eps, kind, scale, diag, rng_mode=1, threads=None):
    if threads is None:
        threads = os.cpu_count() or 1
    return _Params(ndim, nmax, dprime, kind, eps, scale, diag, rng_mode, threads)


class OracleHODLR:
    """CPU restatement of HODLRdD_matrix: build (tree, lists, ACA, leaf blocks),
    matvec and GMRES solve, all in the caller's point order."""

    def __init__(self, pts, lo, hi, *, nmax, dprime, eps, kind, scale, diag, rng_mode=1, threads=None,
                 with_operators=True):
        self.pts = np.ascontiguousarray(pts, dtype=np.float64)
        self.n, self.ndim = self.pts.shape
        self.p = make_params(self.ndim, nmax, dprime, eps, kind, scale, diag, rng_mode, threads)
        lo = np.ascontiguousarray(lo, dtype=np.float64)
        hi = np.ascontiguousarray(hi, dtype=np.float64)
        self.h = lib().orc_build(ctypes.byref(self.p), _d(self.pts), self.n, _d(lo), _d(hi), int(with_operators))
        if not self.h:
            raise ValueError("orc_build rejected its arguments")

    def __del__(self):
        h = getattr(self, "h", None)
        if h:
            lib().orc_free(h)
            self.h = None

    def structure(self):
        L = lib()
        sz = np.zeros(3, np.int64)
        L.orc_structure_sizes(self.h, _q(sz))
        counts = np.zeros(sz[0], np.int64)
        nbr_ptr = np.zeros(sz[0] + 1, np.int64)
        intr_ptr = np.zeros(sz[0] + 1, np.int64)
        nbr = np.zeros(max(sz[1], 1), np.int64)
        intr = np.zeros(max(sz[2], 1), np.int64)
        perm = np.zeros(self.n, np.int64)
        L.orc_get_structure(self.h, _q(counts), _q(nbr_ptr), _q(nbr), _q(intr_ptr), _q(intr), _q(perm))
        levels = [L.orc_level_size(self.h, l) for l in range(L.orc_num_levels(self.h))]
        return dict(level_sizes=np.array(levels, np.int64), node_counts=counts, nbr_ptr=nbr_ptr,
                    nbr=nbr[:sz[1]], intr_ptr=intr_ptr, intr=intr[:sz[2]], leaf_perm=perm)

    def blocks(self):
        L = lib()
        nb = L.orc_num_blocks(self.h)
        a = [np.zeros(nb, np.int64) for _ in range(5)]
        L.orc_get_blocks(self.h, *[_q(x) for x in a])
        return dict(level=a[0], t=a[1], s=a[2], rank=a[3], dense=a[4])

    def block_factors(self, b, m, n, rank):
        U = np.zeros(m * rank, np.float64)
        V = np.zeros(n * rank, np.float64)
        lib().orc_get_block_factors(self.h, b, _d(U), _d(V))
        return U.reshape(rank, m).T, V.reshape(rank, n).T

    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.zeros(self.n, np.float64)
        lib().orc_matvec(self.h, _d(x), _d(y))
        return y

    def solve(self, b, restart=100, max_iter=0, tol=None, x0=None):
        """iterSolver::GMRES as HODLRdD_matrix::solve calls it: x0 = b by default."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.array(b if x0 is None else x0, dtype=np.float64)
        res = np.zeros(1)
        it = lib().orc_gmres(self.h, _d(b), _d(x), restart, max_iter,
                             self.p.eps if tol is None else tol, _d(res))
        return x, int(it), float(res[0])

    def stats(self):
        out = np.zeros(5)
        lib().orc_stats(self.h, _d(out))
        return dict(n_flop=out[0], max_rank=int(out[1]), t_tree=out[2], t_init=out[3], t_matvec=out[4])


def dense_matvec(pts, x, *, kind, scale, diag, rows=None, threads=None):
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n, ndim = pts.shape
    p = make_params(ndim, 1, 0, 0.0, kind, scale, diag, 1, threads)
    x = np.ascontiguousarray(x, dtype=np.float64)
    if rows is None:
        y = np.zeros(n)
        lib().orc_dense_matvec(ctypes.byref(p), _d(pts), n, _d(x), None, 0, _d(y))
    else:
        rows = np.ascontiguousarray(rows, dtype=np.int64)
        y = np.zeros(len(rows))
        lib().orc_dense_matvec(ctypes.byref(p), _d(pts), n, _d(x), _q(rows), len(rows), _d(y))
    return y


def dense_gmres(pts, b, *, kind, scale, diag, restart=100, max_iter=0, tol=1e-10):
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    n, ndim = pts.shape
    p = make_params(ndim, 1, 0, 0.0, kind, scale, diag, 1, 1)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = b.copy()
    res = np.zeros(1)
    it = lib().orc_dense_gmres(ctypes.byref(p), _d(pts), n, _d(b), _d(x), restart, max_iter, tol, _d(res))
    return x, int(it), float(res[0])


def block_seed(level, t, s):
    return int(lib().orc_block_seed(level, t, s))
