"""Several right-hand sides on the tensor cores (hodlr_matvec_tc_device):
BF16 far factors as stored, the right-hand sides split into BF16 high and low
parts, the FP64 near field in three BF16 terms, FP32 accumulation in tensor
memory.  Checked against the same stored operator applied one column at a
time with FP64 vectors (compensated products): the two differ by the
splitting and the FP32 sums, about 1e-5 relative -- far below the BF16
storage error (about 1e-3) that separates both from the FP64 operator, which
must stay as it is."""
import numpy as np
import pytest

from hodlrnd_gb300.kernels import Kernel
from hodlrnd_gb300.matrix import HODLRdD_matrix

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("ndim,n,nmax,dprime,kind,nrhs", [(4, 8192, 128, 0, "inv_r2", 70), (3, 20000, 64, 0, "inv_r", 64),
                                                           (2, 12000, 64, -1, "log_r", 5)])
def test_tc_matvec_matches_the_stored_operator(ndim, n, nmax, dprime, kind, nrhs):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(ndim * 100 + nrhs)
    pts = rng.uniform(0.0, 1.0, (n, ndim))
    scale = 1.0 / n ** ((ndim - 1) / ndim)
    box = ([0.0] * ndim, [1.0] * ndim)
    kw = dict(Nmax=nmax, eps_ACA=1e-4, INTERACTION_TYPE_ALLOWED=dprime)
    Mb = HODLRdD_matrix(Kernel(kind, scale, 1.0), pts, *box, precision="bf16_factors", fp64_check=False,
                        **kw).Assemble_matrix_operators()
    M64 = HODLRdD_matrix(Kernel(kind, scale, 1.0), pts, *box, **kw).Assemble_matrix_operators()
    X = rng.standard_normal((n, nrhs))
    Xd = torch.tensor(X.T.copy(), dtype=torch.float32, device="cuda")  # column major n x nrhs
    Yd = torch.zeros_like(Xd)
    Mb.matvec_tc_device(Xd.data_ptr(), Yd.data_ptr(), nrhs)
    Y = Yd.cpu().numpy().astype(np.float64).T
    Xf = Xd.cpu().numpy().astype(np.float64).T  # the FP32 inputs the tensor path saw
    for k in range(nrhs):
        yb = Mb * Xf[:, k]
        y64 = M64 * Xf[:, k]
        assert rel(Y[:, k], yb) <= 5e-5
        # the distance to the FP64 operator is the BF16 storage's, unchanged
        assert rel(Y[:, k], y64) <= 1.05 * rel(yb, y64) + 5e-5
    Mb.close()
    M64.close()
