"""Request loop (serving) through the C ABI's hodlr_server_* entry points.

A Server owns worker threads ("slots") that admit queued solve requests by
their predicted device bytes against a memory budget, keep keyed geometries
resident on the device (least recently used evicted first) and run requests
concurrently, one CUDA stream per geometry.  The reference has no
counterpart: it builds and solves one HODLRdD_matrix at a time
(HODLRnD include/HDD_matrix.hpp:20-62).

    srv = Server(slots=4, memory_budget_bytes=150 << 30)
    t = srv.submit(points, b, kernel=Kernel("inv_r", s, 1.0), box=(lo, hi), key=7, eps_ACA=1e-8)
    x, info = srv.wait(t)
"""
import ctypes

import numpy as np

from . import _lib


class HodlrServerParams(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("slots", ctypes.c_int32), ("memory_budget_bytes", ctypes.c_uint64),
                ("simulate", ctypes.c_int32), ("reserved", ctypes.c_int32)]


class HodlrRequest(ctypes.Structure):
    _fields_ = [("geometry_key", ctypes.c_uint64), ("params", _lib.HodlrParams), ("kernel", _lib.HodlrKernelDesc),
                ("points", ctypes.c_void_p), ("box_lo", ctypes.c_void_p), ("box_hi", ctypes.c_void_p),
                ("n", ctypes.c_int64), ("b", ctypes.c_void_p), ("nrhs", ctypes.c_int64)]


class HodlrResult(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("built", ctypes.c_int32), ("iterations", ctypes.c_int64),
                ("rel_residual", ctypes.c_double), ("t_queue_s", ctypes.c_double), ("t_build_s", ctypes.c_double),
                ("t_solve_s", ctypes.c_double), ("t_total_s", ctypes.c_double),
                ("predicted_bytes", ctypes.c_uint64), ("actual_bytes", ctypes.c_uint64),
                ("predicted_build_bytes", ctypes.c_uint64), ("t_device_start_s", ctypes.c_double),
                ("t_device_end_s", ctypes.c_double), ("message", ctypes.c_char * 128)]

    def as_dict(self):
        d = {k: getattr(self, k) for k, _ in self._fields_ if k != "message"}
        d["message"] = self.message.decode(errors="replace")
        return d


class HodlrServerStats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_uint64) for k in ("submitted", "completed", "rejected", "builds", "resident_hits",
                                               "evictions", "rhs_solved")] + \
               [(k, ctypes.c_int64) for k in ("queued", "running", "resident")] + [("used_bytes", ctypes.c_uint64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_bound = False


def _bind():
    global _bound
    L = _lib.lib()
    if _bound:
        return L
    P = ctypes.c_void_p
    L.hodlr_server_create.argtypes = [ctypes.POINTER(HodlrServerParams), ctypes.POINTER(P)]
    L.hodlr_server_submit.argtypes = [P, ctypes.POINTER(HodlrRequest), ctypes.POINTER(ctypes.c_uint64)]
    L.hodlr_server_wait.argtypes = [P, ctypes.c_uint64, ctypes.c_double, ctypes.c_void_p, ctypes.POINTER(HodlrResult)]
    L.hodlr_server_stats_get.argtypes = [P, ctypes.POINTER(HodlrServerStats)]
    L.hodlr_server_destroy.argtypes = [P]
    L.hodlr_predict_bytes.argtypes = [ctypes.POINTER(_lib.HodlrParams), ctypes.c_void_p, ctypes.c_int64,
                                      ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_uint64)]
    for f in ("hodlr_server_create", "hodlr_server_submit", "hodlr_server_wait", "hodlr_server_stats_get",
              "hodlr_server_destroy", "hodlr_predict_bytes"):
        getattr(L, f).restype = ctypes.c_int
    _bound = True
    return L


def make_params(ndim, Nmax=64, eps_ACA=1e-10, INTERACTION_TYPE_ALLOWED=0, precision="fp64", restart=100, tol=None,
                max_iter=0, inner_tol=0.0, max_outer=0, ortho="auto", relax=True, relax_below=0.0,
                stored_margin=0.0, fp64_check=True):
    L = _lib.lib()
    p = _lib.HodlrParams()
    L.hodlr_params_default(ctypes.byref(p))
    p.ndim = int(ndim)
    p.nmax = int(Nmax)
    p.dprime = int(INTERACTION_TYPE_ALLOWED)
    p.eps_aca = float(eps_ACA)
    p.restart = int(restart)
    p.tol = float(tol) if tol is not None else 0.0
    p.max_iter = int(max_iter)
    p.precision = {"fp64": _lib.HODLR_PREC_FP64, "mixed": _lib.HODLR_PREC_MIXED,
                   "fp32_factors": _lib.HODLR_PREC_FP32_FACTORS,
                   "bf16_factors": _lib.HODLR_PREC_BF16_FACTORS}[precision]
    p.inner_tol = float(inner_tol)
    p.max_outer = int(max_outer)
    p.ortho = {"auto": _lib.HODLR_ORTHO_AUTO, "mgs": _lib.HODLR_ORTHO_MGS, "cgs2": _lib.HODLR_ORTHO_CGS2}[ortho]
    p.relax = _lib.relax_code(relax)
    p.relax_below = float(relax_below)
    p.stored_margin = float(stored_margin)
    p.fp64_check = _lib.HODLR_FP64_CHECK_AUTO if fp64_check else _lib.HODLR_FP64_CHECK_OFF
    return p


def predict_bytes(points, box, **params):
    """Predicted device bytes of a build and its solves (hodlr_predict_bytes)."""
    L = _bind()
    pts = np.ascontiguousarray(points, dtype=np.float64)
    lo = np.ascontiguousarray(box[0], dtype=np.float64)
    hi = np.ascontiguousarray(box[1], dtype=np.float64)
    p = make_params(pts.shape[1], **params)
    out = ctypes.c_uint64(0)
    _lib.check(L.hodlr_predict_bytes(ctypes.byref(p), pts.ctypes.data, pts.shape[0], lo.ctypes.data, hi.ctypes.data,
                                     ctypes.byref(out)))
    return int(out.value)


class Server:
    def __init__(self, slots=4, memory_budget_bytes=0, device=0, simulate=False):
        L = _bind()
        sp = HodlrServerParams(device=int(device), slots=int(slots), memory_budget_bytes=int(memory_budget_bytes),
                               simulate=1 if simulate else 0)
        self._h = ctypes.c_void_p()
        _lib.check(L.hodlr_server_create(ctypes.byref(sp), ctypes.byref(self._h)))
        self._shapes = {}

    def submit(self, points, b, kernel, box=None, key=0, ndim=None, **params):
        """Queue a solve; returns a ticket.  points=None reuses the resident
        geometry `key` (then ndim must be given)."""
        L = _bind()
        B = np.asarray(b, dtype=np.float64)
        nrhs = 1 if B.ndim == 1 else B.shape[1]
        Bc = np.asfortranarray(B.reshape(B.shape[0], nrhs))
        n = Bc.shape[0]
        req = HodlrRequest()
        req.geometry_key = int(key)
        keep = [Bc]
        if points is not None:
            pts = np.ascontiguousarray(points, dtype=np.float64)
            if pts.shape[0] != n:
                raise ValueError("points and right-hand sides disagree on N")
            ndim = pts.shape[1]
            lo = np.ascontiguousarray(box[0], dtype=np.float64)
            hi = np.ascontiguousarray(box[1], dtype=np.float64)
            keep += [pts, lo, hi]
            req.points, req.box_lo, req.box_hi = pts.ctypes.data, lo.ctypes.data, hi.ctypes.data
        elif ndim is None:
            raise ValueError("ndim is needed when points is None")
        req.params = make_params(ndim, **params)
        req.kernel = _lib.HodlrKernelDesc(kind=kernel.kind, scale=kernel.scale, diag=kernel.diag)
        req.n = n
        req.b = Bc.ctypes.data
        req.nrhs = nrhs
        t = ctypes.c_uint64(0)
        _lib.check(L.hodlr_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        self._shapes[t.value] = (n, nrhs, B.ndim)
        return int(t.value)

    def wait(self, ticket, timeout=-1.0):
        """(x, result dict) when the request finishes; raises HodlrError on a
        failure other than non-convergence, TimeoutError on timeout."""
        L = _bind()
        n, nrhs, nd = self._shapes[ticket]
        x = np.empty((n, nrhs), dtype=np.float64, order="F")
        r = HodlrResult()
        rc = L.hodlr_server_wait(self._h, ticket, float(timeout), x.ctypes.data, ctypes.byref(r))
        if rc == _lib.HODLR_ERR_TIMEOUT:
            raise TimeoutError(f"request {ticket} has not finished")
        del self._shapes[ticket]
        res = r.as_dict()
        if rc not in (_lib.HODLR_OK, _lib.HODLR_ERR_NOT_CONVERGED):
            raise _lib.HodlrError(rc, res["message"] or _lib.last_error())
        return (x[:, 0].copy() if nd == 1 else x), res

    def stats(self):
        s = HodlrServerStats()
        _lib.check(_bind().hodlr_server_stats_get(self._h, ctypes.byref(s)))
        return s.as_dict()

    def close(self):
        if self._h:
            _bind().hodlr_server_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
