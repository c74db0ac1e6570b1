"""User kernels: the device-evaluable counterpart of the reference's user
kernel classes (HODLRnD include/user_kernel.hpp).

The reference asks a kernel class for `getMatrixEntry(i, j)` and
`get_points(...)`.  The GPU engine cannot call back into host code per
entry, so a kernel here also describes itself with `gpu_kernel_desc()`:
(kind, scale, diag) with A_ij = f(|x_i - x_j|) for i != j and A_ii = diag.
`getMatrixEntry` stays available (evaluated on the host with numpy) for
checking and for small dense references.
"""
import math

import numpy as np

from . import _lib

KINDS = {"inv_r": _lib.HODLR_KERNEL_INV_R, "inv_r2": _lib.HODLR_KERNEL_INV_R2,
         "log_r": _lib.HODLR_KERNEL_LOG_R, "exp_neg_r": _lib.HODLR_KERNEL_EXP_NEG_R}


class Kernel:
    """A_ij = scale * g(r_ij) with g in {1/r, 1/r^2, log r, exp(-r)}; A_ii = diag."""

    def __init__(self, kind, scale=1.0, diag=0.0, gridPoints=None):
        self.kind = KINDS[kind] if isinstance(kind, str) else int(kind)
        self.scale = float(scale)
        self.diag = float(diag)
        self.gridPoints = None if gridPoints is None else np.ascontiguousarray(gridPoints, dtype=np.float64)

    def gpu_kernel_desc(self):
        return (self.kind, self.scale, self.diag)

    def get_points(self):
        return self.gridPoints

    def _f(self, d2):
        r = np.sqrt(d2)
        if self.kind == _lib.HODLR_KERNEL_INV_R:
            return self.scale / r
        if self.kind == _lib.HODLR_KERNEL_INV_R2:
            return self.scale / d2
        if self.kind == _lib.HODLR_KERNEL_LOG_R:
            return self.scale * np.log(r)
        return self.scale * np.exp(-r)

    def getMatrixEntry(self, i, j):
        if i == j:
            return self.diag
        d = self.gridPoints[i] - self.gridPoints[j]
        return float(self._f(np.dot(d, d)))

    def getMatrix(self, rows, cols):
        """Dense block A(rows, cols) (kernel_function::getMatrix, include/kernel_function.hpp:43-53)."""
        P = self.gridPoints
        rows = np.asarray(rows)
        cols = np.asarray(cols)
        d2 = np.zeros((len(rows), len(cols)))
        for k in range(P.shape[1]):
            t = P[rows, k][:, None] - P[cols, k][None, :]
            d2 += t * t
        with np.errstate(divide="ignore", invalid="ignore"):
            A = self._f(d2)
        A[rows[:, None] == cols[None, :]] = self.diag
        return A


def _uniform_nodes(a, b, n):
    # include/myHeaders.hpp:111-120
    return np.array([a + (b - a) / float(n - 1) * k for k in range(n)])


def _tensor_grid(ndim, num_points):
    nodes = _uniform_nodes(-1.0, 1.0, num_points)
    g = np.stack(np.meshgrid(*([nodes] * ndim), indexing="ij"), axis=-1)
    return g.reshape(-1, ndim)


class kernel_2d_test(Kernel):
    """-log(r) / (2 pi), A_ii = 0, on a numPoints^2 grid over [-1,1]^2 (include/user_kernel.hpp:10-60)."""

    def __init__(self, numPoints=10):
        super().__init__("log_r", -1.0 / (2 * math.pi), 0.0, _tensor_grid(2, numPoints))


class kernel_3d_test(Kernel):
    """1 / (4 pi r), A_ii = 0, on a numPoints^3 grid over [-1,1]^3 (include/user_kernel.hpp:62-115)."""

    def __init__(self, numPoints=10):
        super().__init__("inv_r", 1.0 / (4 * math.pi), 0.0, _tensor_grid(3, numPoints))


def _kernel4d_diag(h):
    """1 + 32-point Gauss-Legendre quadrature of -exp(-|t|)/(4 pi) over [0, h/2]^4
    (include/user_kernel.hpp:127-131, integral_equation_4D/integral4d.hpp:18-61)."""
    nodes, w = np.polynomial.legendre.leggauss(32)
    half = 0.25 * h
    t = half * nodes + half
    T = np.stack(np.meshgrid(t, t, t, t, indexing="ij"), axis=-1)
    W = w[:, None, None, None] * w[None, :, None, None] * w[None, None, :, None] * w[None, None, None, :]
    return 1.0 + float(np.sum(W * (-1.0 / (4 * math.pi)) * np.exp(-np.sqrt(np.sum(T * T, axis=-1))))) * half ** 4


class kernel_4d_test(Kernel):
    """h^4 (-1/(4 pi)) exp(-r), h = 1/numPoints, A_ii = 1 + the quadrature above, on a
    numPoints^4 grid over [-1,1]^4 (include/user_kernel.hpp:117-179)."""

    def __init__(self, numPoints=10):
        h = 1.0 / numPoints
        super().__init__("exp_neg_r", h ** 4 * (-1.0 / (4 * math.pi)), _kernel4d_diag(h), _tensor_grid(4, numPoints))
