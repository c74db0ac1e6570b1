"""The C++ drop-in facade (include/hodlrnd_matrix.hpp) as a HODLRnD user
would use it: the complete program in INTEGRATION.md's C++ block is extracted
as it stands, compiled with g++ against include/ and linked to
libhodlrnd_gb300.so.  On the CPU the test only compiles and links it; on the
GPU it runs the program (reference argument shapes: std::vector<ptsnD>*,
box vectors, Kmat * x, Kmat.solve(b)) and checks its matvec and solve against
the Python path on the same points, which calls the same C ABI: the results
must be identical bit for bit.
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "hodlrnd_gb300")


def _snippet():
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    sec = text[text.index("## The binding a HODLRnD user adds (C++)"):]
    m = re.search(r"```cpp\n(.*?)```", sec, re.S)
    assert m, "INTEGRATION.md has no C++ block in its binding section"
    return m.group(1)


def _compile(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    if not os.path.exists(os.path.join(LIBDIR, "libhodlrnd_gb300.so")):
        pytest.skip("libhodlrnd_gb300.so not built")
    src = tmp_path / "main.cpp"
    src.write_text(_snippet())
    exe = tmp_path / "facade_main"
    cmd = ["g++", "-std=c++17", "-Wall", "-Werror", "-I" + os.path.join(ROOT, "include"), str(src), "-o", str(exe),
           "-L" + LIBDIR, "-lhodlrnd_gb300", "-Wl,-rpath," + LIBDIR]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_facade_snippet_compiles_and_links(tmp_path):
    _compile(tmp_path)


@pytest.mark.gpu
def test_facade_snippet_matches_python_path(tmp_path):
    from hodlrnd_gb300 import storedata
    from hodlrnd_gb300.kernels import Kernel
    from hodlrnd_gb300.matrix import HODLRdD_matrix

    exe = _compile(tmp_path)
    n = 6000
    rng = np.random.default_rng(31)
    pts = rng.uniform(0.0, 1.0, (n, 3))
    x = rng.standard_normal(n)
    storedata.save_vec(str(tmp_path / "points.bin"), pts.reshape(-1))
    storedata.save_vec(str(tmp_path / "x.bin"), x)
    r = subprocess.run([str(exe), str(tmp_path / "points.bin"), str(tmp_path / "x.bin"), str(tmp_path / "b.bin"),
                        str(tmp_path / "y.bin")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Maximum rank across the Tree" in r.stdout
    b_cpp = storedata.load_vec(str(tmp_path / "b.bin"))
    y_cpp = storedata.load_vec(str(tmp_path / "y.bin"))
    M = HODLRdD_matrix(Kernel("inv_r", 1.0 / n ** (2.0 / 3.0), 1.0), pts, [0.0] * 3, [1.0] * 3, Nmax=64,
                       eps_ACA=1e-8, INTERACTION_TYPE_ALLOWED=0).Assemble_matrix_operators()
    b = M * x
    y = M.solve(b)
    assert M.last_solve["converged"] == 1
    assert np.array_equal(b_cpp, b)
    assert np.array_equal(y_cpp, y)
    assert np.linalg.norm(y - x) / np.linalg.norm(x) < 1e-6
    M.close()
