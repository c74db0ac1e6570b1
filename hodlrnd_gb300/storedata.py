"""Vector files in the format of HODLRnD's storedata::load_vec / save_vec
(include/myHeaders.hpp:146-170), through the C ABI's hodlr_vec_load /
hodlr_vec_save: a cereal PortableBinary archive of one std::vector<double>
(1-byte endianness tag, u64 count, float64 values), read and written without
cereal.  The reference's functions take and return Eigen::VectorXd; these take
and return 1-D float64 numpy arrays."""
import ctypes
import os

import numpy as np

from . import _lib

_D = ctypes.POINTER(ctypes.c_double)


def load_vec(fname):
    """storedata::load_vec(std::string fname) (include/myHeaders.hpp:150-159)."""
    L = _lib.lib()
    path = os.fsencode(fname)
    n = ctypes.c_int64(0)
    _lib.check(L.hodlr_vec_load(path, None, 0, ctypes.byref(n)))
    x = np.empty(n.value, dtype=np.float64)
    _lib.check(L.hodlr_vec_load(path, x.ctypes.data_as(_D), n.value, ctypes.byref(n)))
    return x


def save_vec(fname, X):
    """storedata::save_vec(std::string fname, Eigen::VectorXd X) (include/myHeaders.hpp:161-168)."""
    x = np.ascontiguousarray(X, dtype=np.float64).reshape(-1)
    _lib.check(_lib.lib().hodlr_vec_save(os.fsencode(fname), x.ctypes.data_as(_D), x.size))
