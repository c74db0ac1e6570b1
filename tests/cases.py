"""Seeded parity cases shared by the fixture generator and the tests.

Each case names the reference hyper-parameters (NDIM, Nmax, d' =
INTERACTION_TYPE_ALLOWED, eps_ACA; include/myHeaders.hpp:35-48), the kernel
(kind, scale, diagonal) and how its points and vectors are drawn.  Points are
i.i.d. uniform in the box from numpy's PCG64 with the case seed; fixtures also
store the points themselves, so a change in numpy's streams cannot move them.
"""
import numpy as np

INV_R, INV_R2, LOG_R, EXP_NEG_R = 1, 2, 3, 4

# Cases compared against the reference's own headers compiled in place.  None of
# them has an empty node with a non-empty far partner: the reference's matvec
# dereferences an unallocated block array there (include/HDD_node.hpp:120-131
# allocate LR only for non-empty nodes, :243-250 read it for every node).
REF_CASES = {
    # config 1 (HODLR2D, CPU-runnable case) at full size
    "c1_2d_n10000": dict(ndim=2, n=10000, nmax=64, dprime=0, eps=1e-10, kind=INV_R,
                         scale=1.0 / 10000, diag=1.0, lo=-1.0, hi=1.0, seed=1),
    "c1_2d_n2000": dict(ndim=2, n=2000, nmax=64, dprime=0, eps=1e-10, kind=INV_R,
                        scale=1.0 / 2000, diag=1.0, lo=-1.0, hi=1.0, seed=2),
    "hodlr3d_n4096": dict(ndim=3, n=4096, nmax=64, dprime=0, eps=1e-8, kind=INV_R,
                          scale=1.0 / 4096 ** (2.0 / 3.0), diag=1.0, lo=0.0, hi=1.0, seed=4),
    "edge3d_exp_n3000": dict(ndim=3, n=3000, nmax=64, dprime=1, eps=1e-6, kind=EXP_NEG_R,
                             scale=1.0 / 3000 ** (2.0 / 3.0), diag=1.0, lo=0.0, hi=1.0, seed=8),
    "hmat2d_log_n3000": dict(ndim=2, n=3000, nmax=50, dprime=-1, eps=1e-8, kind=LOG_R,
                             scale=-1.0 / (2 * np.pi) / 3000 ** 0.5, diag=1.0, lo=0.0, hi=1.0, seed=5),
    "hmat4d_invr2_n2048": dict(ndim=4, n=2048, nmax=128, dprime=-1, eps=1e-8, kind=INV_R2,
                               scale=1.0 / 2048 ** 0.5, diag=1.0, lo=0.0, hi=1.0, seed=6),
}

# kernel_4d_test on its numPoints = 10 tensor grid (include/user_kernel.hpp:117-179)
# with the reference's shipped hyper-parameters (include/myHeaders.hpp:35-47).
GOLDEN4D = dict(ndim=4, nmax=1000, dprime=1, eps=1e-10, num_points=10)


def points(case):
    rng = np.random.default_rng(case["seed"])
    return rng.uniform(case["lo"], case["hi"], (case["n"], case["ndim"]))


def vectors(case):
    """(x, b): x drawn uniform in [-1, 1]; b is drawn independently (N(0,1))."""
    rng = np.random.default_rng(1000 + case["seed"])
    x = rng.uniform(-1.0, 1.0, case["n"])
    b = rng.standard_normal(case["n"])
    return x, b


def box(case):
    return [case["lo"]] * case["ndim"], [case["hi"]] * case["ndim"]


def grid4d(num_points=10):
    """kernel_4d_test's grid: uniform_nodes(-1, 1, n) per axis, (i, j, k, l)
    lexicographic (include/user_kernel.hpp:142-161, include/myHeaders.hpp:111-120)."""
    nodes = np.array([-1.0 + 2.0 / (num_points - 1) * k for k in range(num_points)])
    g = np.stack(np.meshgrid(nodes, nodes, nodes, nodes, indexing="ij"), axis=-1)
    return g.reshape(-1, 4)


def kernel4d_test_params(num_points=10):
    """(scale, diag) of kernel_4d_test: h^4 * (-1/(4 pi)) e^{-r}, h = 1/numPoints,
    diag = 1 + the 32-point Gauss-Legendre quadrature of -e^{-|t|}/(4 pi) over
    [0, h/2]^4 (user_kernel.hpp:117-131, integral_equation_4D/integral4d.hpp:18-61)."""
    h = 1.0 / num_points
    c = -1.0 / (4 * np.pi)
    nodes, weights = np.polynomial.legendre.leggauss(32)
    half = 0.5 * (h / 2)
    t = half * nodes + half
    w = weights
    T = np.stack(np.meshgrid(t, t, t, t, indexing="ij"), axis=-1)
    W = w[:, None, None, None] * w[None, :, None, None] * w[None, None, :, None] * w[None, None, None, :]
    integral = np.sum(W * c * np.exp(-np.sqrt(np.sum(T * T, axis=-1)))) * half ** 4
    return h ** 4 * c, 1.0 + integral
