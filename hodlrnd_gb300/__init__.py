"""GB300-native HODLRnD engine: the reference's HODLR build / matvec / GMRES
path (HODLRnD, include/HDD_matrix.hpp) on hand-written sm_103a kernels behind
the C ABI of include/hodlrnd.h."""
from ._lib import HodlrError, lib  # noqa: F401
from .kernels import Kernel, kernel_2d_test, kernel_3d_test, kernel_4d_test  # noqa: F401
from .matrix import HODLRdD_matrix  # noqa: F401
from .storedata import load_vec, save_vec  # noqa: F401
