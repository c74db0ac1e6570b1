"""Test-oracle only: readers/writers for the oracle's binary formats.

* `read_named_arrays(path)` reads the named-array dump written by
  oracle/ref_driver.cpp (u32 name length, name, 1-byte dtype code 'd'|'q',
  u64 count, raw little-endian data).
* `read_cereal_vector(path)` reads a cereal PortableBinary std::vector<double>
  as stored by HODLRnD's storedata::save_vec (include/myHeaders.hpp:162-168):
  one endianness byte (1 = little endian), a u64 element count, then the
  float64 payload.
* `write_driver_input(...)` writes the input file read by ref_driver.cpp.
"""
import struct

import numpy as np


def read_named_arrays(path):
    out = {}
    with open(path, "rb") as f:
        buf = f.read()
    pos = 0
    while pos < len(buf):
        (ln,) = struct.unpack_from("<I", buf, pos)
        pos += 4
        name = buf[pos:pos + ln].decode()
        pos += ln
        code = chr(buf[pos])
        pos += 1
        (n,) = struct.unpack_from("<Q", buf, pos)
        pos += 8
        dt = {"d": "<f8", "q": "<i8"}[code]
        out[name] = np.frombuffer(buf, dtype=dt, count=n, offset=pos).copy()
        pos += 8 * n
    return out


def read_cereal_vector(path):
    with open(path, "rb") as f:
        buf = f.read()
    if buf[0] != 1:
        raise ValueError("cereal portable binary: big-endian payloads are not supported")
    (n,) = struct.unpack_from("<Q", buf, 1)
    if len(buf) != 9 + 8 * n:
        raise ValueError("cereal portable binary: size mismatch")
    return np.frombuffer(buf, dtype="<f8", count=n, offset=9).copy()


def write_driver_input(path, pts, lo, hi, kind, scale, diag, x, b, restart=100, max_iter=0, tol=1e-10):
    pts = np.ascontiguousarray(pts, dtype="<f8")
    n, ndim = pts.shape
    with open(path, "wb") as f:
        f.write(struct.pack("<qiiddiid", n, ndim, kind, scale, diag, restart, max_iter, tol))
        f.write(pts.tobytes())
        f.write(np.asarray(lo, "<f8").tobytes())
        f.write(np.asarray(hi, "<f8").tobytes())
        f.write(np.asarray(x, "<f8").tobytes())
        f.write(np.asarray(b, "<f8").tobytes())
