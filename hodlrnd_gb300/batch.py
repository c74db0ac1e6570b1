"""Batches of independent HODLR operators (hodlr_build_batch and friends).

All instances share one ACA launch sequence at build time and one merged
plan for matvecs, replayed as a CUDA graph; each instance is also an
ordinary operator for solves.  No counterpart in the reference, which builds
one HODLRdD_matrix at a time (HODLRnD include/HDD_matrix.hpp:20-62)."""
import ctypes

import numpy as np

from . import _lib
from .server import make_params

_bound = False


def _bind():
    global _bound
    L = _lib.lib()
    if _bound:
        return L
    P = ctypes.c_void_p
    L.hodlr_build_batch.argtypes = [P, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p),
                                    ctypes.POINTER(ctypes.c_int64), P, P, ctypes.POINTER(_lib.HodlrKernelDesc),
                                    ctypes.POINTER(P)]
    L.hodlr_batch_offsets.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    L.hodlr_batch_op.argtypes = [P, ctypes.c_int32, ctypes.POINTER(P)]
    L.hodlr_batch_matvec_device.argtypes = [P, P, P, ctypes.c_int64, P]
    L.hodlr_batch_destroy.argtypes = [P]
    for f in ("hodlr_build_batch", "hodlr_batch_offsets", "hodlr_batch_op", "hodlr_batch_matvec_device",
              "hodlr_batch_destroy"):
        getattr(L, f).restype = ctypes.c_int
    _bound = True
    return L


class HODLRdD_batch:
    """count operators: kernels[i] on points_list[i] in boxes[i] = (lo, hi),
    all with the same parameters (HODLRdD_matrix keywords)."""

    def __init__(self, kernels, points_list, boxes, device=0, **params):
        L = _bind()
        pts = [np.ascontiguousarray(p, dtype=np.float64) for p in points_list]
        ndim = pts[0].shape[1]
        p = make_params(ndim, **params)
        p.device = int(device)
        self._ctx = ctypes.c_void_p()
        _lib.check(L.hodlr_ctx_create(ctypes.byref(p), ctypes.byref(self._ctx)))
        count = len(pts)
        ptrs = (ctypes.c_void_p * count)(*[q.ctypes.data for q in pts])
        ns = (ctypes.c_int64 * count)(*[q.shape[0] for q in pts])
        lo = np.ascontiguousarray([b[0] for b in boxes], dtype=np.float64)
        hi = np.ascontiguousarray([b[1] for b in boxes], dtype=np.float64)
        kd = (_lib.HodlrKernelDesc * count)(*[_lib.HodlrKernelDesc(kind=k.kind, scale=k.scale, diag=k.diag)
                                              for k in kernels])
        self._h = ctypes.c_void_p()
        _lib.check(L.hodlr_build_batch(self._ctx, count, ptrs, ns, lo.ctypes.data, hi.ctypes.data, kd,
                                       ctypes.byref(self._h)), self._ctx)
        off = np.zeros(count + 1, dtype=np.int64)
        _lib.check(L.hodlr_batch_offsets(self._h, off.ctypes.data_as(ctypes.POINTER(ctypes.c_int64))))
        self.offsets = off
        self.count = count
        self.dtype = np.float32 if params.get("precision") == "mixed" else np.float64

    def op(self, i):
        """The raw hodlr_op* of instance i (owned by the batch)."""
        h = ctypes.c_void_p()
        _lib.check(_bind().hodlr_batch_op(self._h, int(i), ctypes.byref(h)), self._ctx)
        return h

    def matvec_device(self, d_x, d_y, nrhs, stream):
        _lib.check(_bind().hodlr_batch_matvec_device(self._h, d_x, d_y, int(nrhs), stream), self._ctx)

    def close(self):
        L = _bind()
        if self._h:
            L.hodlr_batch_destroy(self._h)
            self._h = ctypes.c_void_p()
        if self._ctx:
            L.hodlr_ctx_destroy(self._ctx)
            self._ctx = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
