"""Vector files (hodlr_vec_load / hodlr_vec_save, storedata.load_vec/save_vec)
in the reference's cereal portable-binary format (HODLRnD
include/myHeaders.hpp:146-170).  CPU only.

Pinned byte for byte against the reference's own files data/x_10000.bin and
data/rhs_10000.bin: saving their values (tests/golden/golden_kernel4d_n10000.npz)
must give files with the SHA-256 recorded from the originals
(tests/golden/ref_vec_files.json, made by tests/golden/make_golden.py)."""
import hashlib
import json
import os
import struct

import numpy as np
import pytest

from hodlrnd_gb300 import _lib
from hodlrnd_gb300.storedata import load_vec, save_vec

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module", autouse=True)
def built_library():
    if not os.path.exists(_lib.LIB_PATH):
        from hodlrnd_gb300 import build
        build.build()


@pytest.mark.parametrize("key,name", [("x", "x_10000.bin"), ("rhs", "rhs_10000.bin")])
def test_save_vec_reproduces_reference_files(tmp_path, key, name):
    g = np.load(os.path.join(GOLDEN, "golden_kernel4d_n10000.npz"))
    want = json.load(open(os.path.join(GOLDEN, "ref_vec_files.json")))[name]
    path = tmp_path / name
    save_vec(path, g[key])
    buf = path.read_bytes()
    assert len(buf) == want["bytes"]
    assert hashlib.sha256(buf).hexdigest() == want["sha256"]
    assert np.array_equal(load_vec(path), g[key])


def test_round_trip_and_layout(tmp_path):
    x = np.random.default_rng(1).standard_normal(1000)
    p = tmp_path / "v.bin"
    save_vec(p, x)
    buf = p.read_bytes()
    assert buf[:9] == b"\x01" + struct.pack("<Q", 1000)
    assert buf[9:] == x.astype("<f8").tobytes()
    assert np.array_equal(load_vec(p), x)


def test_empty_vector(tmp_path):
    p = tmp_path / "e.bin"
    save_vec(p, np.zeros(0))
    assert p.read_bytes() == b"\x01" + bytes(8)
    assert load_vec(p).size == 0


def test_big_endian_payload_is_read(tmp_path):
    x = np.array([1.5, -2.25, 3e300, 5e-324])
    p = tmp_path / "be.bin"
    p.write_bytes(b"\x00" + struct.pack(">Q", 4) + x.astype(">f8").tobytes())
    assert np.array_equal(load_vec(p), x)


@pytest.mark.parametrize("blob", [b"", b"\x01\x02", b"\x02" + struct.pack("<Q", 0),
                                  b"\x01" + struct.pack("<Q", 3) + bytes(16),
                                  b"\x01" + struct.pack("<Q", 1) + bytes(16)])
def test_malformed_files_are_rejected(tmp_path, blob):
    p = tmp_path / "bad.bin"
    p.write_bytes(blob)
    with pytest.raises(_lib.HodlrError) as e:
        load_vec(p)
    assert e.value.code == _lib.HODLR_ERR_IO


def test_missing_file_and_small_buffer(tmp_path):
    with pytest.raises(_lib.HodlrError) as e:
        load_vec(tmp_path / "absent.bin")
    assert e.value.code == _lib.HODLR_ERR_IO
    import ctypes

    p = tmp_path / "v.bin"
    save_vec(p, np.arange(10.0))
    buf = np.zeros(5)
    n = ctypes.c_int64(0)
    rc = _lib.lib().hodlr_vec_load(os.fsencode(p), buf.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 5,
                                   ctypes.byref(n))
    assert rc == _lib.HODLR_ERR_INVALID and n.value == 10
