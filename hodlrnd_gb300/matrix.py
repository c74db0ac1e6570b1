"""HODLRdD_matrix: the reference's matrix API over the GPU engine's C ABI.

Mirrors HODLRnD's `HODLRdD_matrix<Kernel>` (include/HDD_matrix.hpp:10-89):
construct from a user kernel, its points and a bounding box (the tree and
interaction lists are built here), `Assemble_matrix_operators()` (ACA of
every admissible block, dense leaf blocks; on the GPU), `*` (matvec),
`solve(b)` (GMRES with x0 = b, restart 100, tol = eps_ACA), `get_size()`,
`print_matrix_details()` and `print_matrix_statistics()`.  The reference's
compile-time constants (include/myHeaders.hpp:35-48) are keyword arguments
with the same names.
"""
import ctypes
import os

import numpy as np

from . import _lib

_D = ctypes.POINTER(ctypes.c_double)
_I64 = ctypes.POINTER(ctypes.c_int64)
_I32 = ctypes.POINTER(ctypes.c_int32)


def _dp(a):
    return a.ctypes.data_as(_D)


class HODLRdD_matrix:
    def __init__(self, userkernel, gridPoints, x1, x2, *, Nmax=64, eps_ACA=1e-10, INTERACTION_TYPE_ALLOWED=0,
                 precision="fp64", restart=100, tol=None, max_iter=0, device=0, device_budget_bytes=0, rank_cap=0,
                 inner_tol=0.0, max_outer=0, ortho="auto", relax=True, relax_below=0.0, stored_margin=0.0,
                 fp64_check=True):
        self.kernel = userkernel
        self.points = np.ascontiguousarray(gridPoints, dtype=np.float64)
        if self.points.ndim != 2:
            raise ValueError("gridPoints must be an (N, NDIM) array")
        self.N, self.NDIM = self.points.shape
        self.x1 = np.ascontiguousarray(x1, dtype=np.float64).reshape(-1)
        self.x2 = np.ascontiguousarray(x2, dtype=np.float64).reshape(-1)
        if self.x1.size != self.NDIM or self.x2.size != self.NDIM:
            raise ValueError("the bounding box must have NDIM entries per corner")
        L = _lib.lib()
        p = _lib.HodlrParams()
        L.hodlr_params_default(ctypes.byref(p))
        p.ndim = self.NDIM
        p.nmax = int(Nmax)
        p.dprime = int(INTERACTION_TYPE_ALLOWED)
        p.eps_aca = float(eps_ACA)
        p.restart = int(restart)
        p.tol = float(tol) if tol is not None else 0.0
        p.max_iter = int(max_iter)
        p.precision = {"fp64": _lib.HODLR_PREC_FP64, "mixed": _lib.HODLR_PREC_MIXED,
                       "fp32_factors": _lib.HODLR_PREC_FP32_FACTORS,
                       "bf16_factors": _lib.HODLR_PREC_BF16_FACTORS}[precision]
        p.device = int(device)
        p.device_budget_bytes = int(device_budget_bytes)
        p.rank_cap = int(rank_cap)
        p.inner_tol = float(inner_tol)
        p.max_outer = int(max_outer)
        p.ortho = {"auto": _lib.HODLR_ORTHO_AUTO, "mgs": _lib.HODLR_ORTHO_MGS, "cgs2": _lib.HODLR_ORTHO_CGS2}[ortho]
        p.relax = _lib.relax_code(relax)
        p.relax_below = float(relax_below)
        p.stored_margin = float(stored_margin)
        p.fp64_check = _lib.HODLR_FP64_CHECK_AUTO if fp64_check else _lib.HODLR_FP64_CHECK_OFF
        self.params = p
        self._ctx = None
        self._op = None
        self.last_solve = None
        # Tree and interaction lists (Tree::Tree, include/HDD_tree.hpp:23-74) -- host only
        tree = ctypes.c_void_p()
        _lib.check(L.hodlr_tree_build(ctypes.byref(p), _dp(self.points), self.N, _dp(self.x1), _dp(self.x2),
                                      ctypes.byref(tree)))
        self._tree = tree

    # ------------------------------------------------------------ lifecycle
    def close(self):
        L = _lib.lib()
        if self._op:
            L.hodlr_op_destroy(self._op)
            self._op = None
        if self._ctx:
            L.hodlr_ctx_destroy(self._ctx)
            self._ctx = None
        if self._tree:
            L.hodlr_tree_destroy(self._tree)
            self._tree = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def get_size(self):
        return self.N

    def Assemble_matrix_operators(self):
        L = _lib.lib()
        if self._ctx is None:
            ctx = ctypes.c_void_p()
            _lib.check(L.hodlr_ctx_create(ctypes.byref(self.params), ctypes.byref(ctx)))
            self._ctx = ctx
        if self._op is not None:
            L.hodlr_op_destroy(self._op)
            self._op = None
        kind, scale, diag = self.kernel.gpu_kernel_desc()
        kd = _lib.HodlrKernelDesc(int(kind), 0, float(scale), float(diag))
        op = ctypes.c_void_p()
        _lib.check(L.hodlr_build(self._ctx, _dp(self.points), self.N, _dp(self.x1), _dp(self.x2), ctypes.byref(kd),
                                 ctypes.byref(op)), self._ctx)
        self._op = op
        return self

    # ------------------------------------------------------------ files
    def save(self, path):
        """Write the built operator to `path` (hodlr_op_save): parameters,
        kernel, points, box, block ranks and the compressed far field."""
        self._need_op()
        _lib.check(_lib.lib().hodlr_op_save(self._op, _dp(self.points), os.fsencode(path)), self._ctx)

    @classmethod
    def load(cls, path, device=0):
        """An operator read back by hodlr_op_load (no ACA) on `device`."""
        L = _lib.lib()
        self = cls.__new__(cls)
        p = _lib.HodlrParams()
        L.hodlr_params_default(ctypes.byref(p))
        p.device = int(device)
        self.params = p
        self._tree = None
        self._op = None
        self.last_solve = None
        self.kernel = None
        self.points = None
        ctx = ctypes.c_void_p()
        _lib.check(L.hodlr_ctx_create(ctypes.byref(p), ctypes.byref(ctx)))
        self._ctx = ctx
        op = ctypes.c_void_p()
        _lib.check(L.hodlr_op_load(self._ctx, os.fsencode(path), ctypes.byref(op)), self._ctx)
        self._op = op
        st = self.statistics()
        self.N = int(st["n"])
        return self

    def _need_op(self):
        if self._op is None:
            raise _lib.HodlrError(_lib.HODLR_ERR_STATE, "call Assemble_matrix_operators() first")

    # ------------------------------------------------------------ operator
    def matvec(self, x):
        """y = A x for x of shape (N,) or (N, nrhs) (host arrays, caller's point order)."""
        self._need_op()
        x = np.asarray(x, dtype=np.float64)
        vec = x.ndim == 1
        X = np.asfortranarray(x.reshape(self.N, -1))
        Y = np.zeros_like(X, order="F")
        _lib.check(_lib.lib().hodlr_matvec(self._op, _dp(X), _dp(Y), X.shape[1]), self._ctx)
        return Y[:, 0] if vec else Y

    def __mul__(self, x):
        return self.matvec(x)

    def matvec_device(self, x_ptr, y_ptr, nrhs=1, stream=0):
        """Device pointers (e.g. torch.Tensor.data_ptr()), asynchronous on `stream`."""
        self._need_op()
        _lib.check(_lib.lib().hodlr_matvec_device(self._op, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr), nrhs,
                                                  ctypes.c_void_p(stream)), self._ctx)

    def matvec_tc_device(self, x_ptr, y_ptr, nrhs, stream=0):
        """Y = A X on the tensor cores (hodlr_matvec_tc_device): BF16 factors,
        FP32 n x nrhs column-major device arrays; synchronises `stream`."""
        self._need_op()
        _lib.check(_lib.lib().hodlr_matvec_tc_device(self._op, ctypes.c_void_p(x_ptr), ctypes.c_void_p(y_ptr),
                                                     int(nrhs), ctypes.c_void_p(stream)), self._ctx)

    def solve(self, b, *, out=None, raise_on_stall=False):
        """x with A x = b (HODLRdD_matrix::solve): FP64 GMRES with x0 = b, or
        FP64 iterative refinement around FP32 GMRES in mixed precision.
        `out` (same shape as b, float64, Fortran order) receives x in place."""
        self._need_op()
        b = np.asarray(b, dtype=np.float64)
        vec = b.ndim == 1
        B = np.asfortranarray(b.reshape(self.N, -1))
        if out is not None:
            X = out.reshape(self.N, -1)
            if X.dtype != np.float64 or not X.flags.f_contiguous:
                raise ValueError("out must be a float64 Fortran-ordered array")
        else:
            X = np.zeros_like(B, order="F")
        info = _lib.HodlrSolveInfo()
        rc = _lib.lib().hodlr_solve(self._op, _dp(B), _dp(X), B.shape[1], ctypes.byref(info))
        self.last_solve = {k: getattr(info, k) for k, _ in info._fields_ if k != "reserved"}
        if rc != _lib.HODLR_OK and (rc != _lib.HODLR_ERR_NOT_CONVERGED or raise_on_stall):
            _lib.check(rc, self._ctx)
        return X[:, 0] if vec else X

    def solve_device(self, b_ptr, x_ptr, nrhs=1, stream=0):
        self._need_op()
        info = _lib.HodlrSolveInfo()
        rc = _lib.lib().hodlr_solve_device(self._op, ctypes.c_void_p(b_ptr), ctypes.c_void_p(x_ptr), nrhs,
                                           ctypes.c_void_p(stream), ctypes.byref(info))
        self.last_solve = {k: getattr(info, k) for k, _ in info._fields_ if k != "reserved"}
        if rc not in (_lib.HODLR_OK, _lib.HODLR_ERR_NOT_CONVERGED):
            _lib.check(rc, self._ctx)
        return self.last_solve

    def set_solver(self, restart=100, tol=None, max_iter=0, inner_tol=0.0, max_outer=0):
        """Solver settings for later solves (iterSolver's arguments, include/GMRES.hpp:56-63)."""
        self._need_op()
        _lib.check(_lib.lib().hodlr_set_solver(self._op, int(restart), float(tol) if tol else 0.0, int(max_iter),
                                               float(inner_tol), int(max_outer)), self._ctx)

    def set_relax(self, relax=True, relax_below=0.0):
        """FP32/BF16-factor solves: relaxed products (True: once the residual allows, False: never,
        "always": every product, FP32 accumulation) and their threshold (0: tol * 1e5)."""
        self._need_op()
        _lib.check(_lib.lib().hodlr_set_relax(self._op, _lib.relax_code(relax),
                                              float(relax_below)), self._ctx)

    # ------------------------------------------------------------ introspection
    def statistics(self):
        self._need_op()
        s = _lib.HodlrStats()
        _lib.check(_lib.lib().hodlr_stats_get(self._op, ctypes.byref(s)))
        return s.as_dict()

    def print_matrix_statistics(self):
        """The figures of print_matrix_statistics (include/HDD_matrix.hpp:69-85)."""
        s = self.statistics()
        print(f"Memory (in GB) : {s['memory_gb']}")
        print(f"Number of FLOP : {s['n_flop']}")
        print(f"Compression Ratio : {s['compression_ratio']}")
        print(f"Maximum rank across the Tree : {s['max_rank']}")
        print(f"Time to Initialize (in s) : {s['t_build_s']}")
        print(f"Matrix-Vector time (in s) : {s['t_matvec_s']}")

    def tree_structure(self, device=False):
        """Tree and lists as arrays.  device=True builds them again on the GPU
        (hodlr_tree_build_device, the path hodlr_build takes) instead of
        returning the host build's."""
        L = _lib.lib()
        if device:
            tree = ctypes.c_void_p()
            _lib.check(L.hodlr_tree_build_device(ctypes.byref(self.params), _dp(self.points), self.N, _dp(self.x1),
                                                 _dp(self.x2), ctypes.byref(tree)))
            try:
                return self._structure(tree)
            finally:
                L.hodlr_tree_destroy(tree)
        return self._structure(self._tree)

    def _structure(self, tree):
        L = _lib.lib()
        sz = np.zeros(6, np.int64)
        _lib.check(L.hodlr_tree_sizes(tree, sz.ctypes.data_as(_I64)))
        levels, nodes = int(sz[0]), int(sz[1])
        out = dict(level_sizes=np.zeros(levels, np.int64), node_counts=np.zeros(nodes, np.int64),
                   nbr_ptr=np.zeros(nodes + 1, np.int64), nbr=np.zeros(max(int(sz[2]), 1), np.int64),
                   intr_ptr=np.zeros(nodes + 1, np.int64), intr=np.zeros(max(int(sz[3]), 1), np.int64),
                   leaf_perm=np.zeros(self.N, np.int64))
        _lib.check(L.hodlr_tree_get(tree, *[out[k].ctypes.data_as(_I64) for k in
                                                 ("level_sizes", "node_counts", "nbr_ptr", "nbr", "intr_ptr",
                                                  "intr", "leaf_perm")]))
        out["nbr"] = out["nbr"][:int(sz[2])]
        out["intr"] = out["intr"][:int(sz[3])]
        out["n_far_blocks"] = int(sz[4])
        out["n_near_blocks"] = int(sz[5])
        return out

    def print_matrix_details(self):
        """Per level: node sizes and list lengths (print_matrix_details, include/HDD_matrix.hpp:63-67)."""
        s = self.tree_structure()
        off = 0
        for l, ls in enumerate(s["level_sizes"]):
            cnt = s["node_counts"][off:off + ls]
            print(f"Level[{l}] nodes={ls} points min/max={cnt.min()}/{cnt.max()}")
            off += ls

    def blocks(self):
        self._need_op()
        nb = self.statistics()["n_far_blocks"]
        lv = np.zeros(nb, np.int32)
        t = np.zeros(nb, np.int64)
        s = np.zeros(nb, np.int64)
        r = np.zeros(nb, np.int32)
        _lib.check(_lib.lib().hodlr_get_blocks(self._op, lv.ctypes.data_as(_I32), t.ctypes.data_as(_I64),
                                               s.ctypes.data_as(_I64), r.ctypes.data_as(_I32)))
        return dict(level=lv, t=t, s=s, rank=r)

    def block(self, b):
        """(U, V, dense) of far block b: U V^T approximates the block (the L, R of
        LowRankMat, include/LowRank_matrix.hpp:10); a dense block comes back as U."""
        self._need_op()
        m, n, r, d = (ctypes.c_int32() for _ in range(4))
        L = _lib.lib()
        _lib.check(L.hodlr_get_block(self._op, int(b), ctypes.byref(m), ctypes.byref(n), ctypes.byref(r),
                                     ctypes.byref(d), None, None))
        if d.value:
            U = np.zeros((n.value, m.value))
            _lib.check(L.hodlr_get_block(self._op, int(b), None, None, None, None, _dp(U), None))
            return U.T.copy(), None, True
        U = np.zeros((r.value, m.value))
        V = np.zeros((r.value, n.value))
        _lib.check(L.hodlr_get_block(self._op, int(b), None, None, None, None, _dp(U), _dp(V)))
        return U.T.copy(), V.T.copy(), False

    def trace(self, on=None):
        """Enable/disable tracing (on=True/False) or read the accumulated figures."""
        self._need_op()
        L = _lib.lib()
        if on is not None:
            _lib.check(L.hodlr_trace_enable(self._op, 1 if on else 0), self._ctx)
            return None
        t = _lib.HodlrTrace()
        _lib.check(L.hodlr_trace_get(self._op, ctypes.byref(t)), self._ctx)
        out = {}
        for k, name in _lib.TRACE_NAMES.items():
            if t.launches[k]:
                out[name] = dict(launches=int(t.launches[k]), total_ms=float(t.total_ms[k]),
                                 bytes_per_launch=float(t.bytes_per_launch[k]))
        return out

    def permutation(self):
        self._need_op()
        p = np.zeros(self.N, np.int64)
        _lib.check(_lib.lib().hodlr_get_permutation(self._op, p.ctypes.data_as(_I64)))
        return p
