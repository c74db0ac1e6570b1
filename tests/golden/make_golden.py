"""Generate the parity fixtures in tests/golden/ from the reference itself.

Run where the HODLRnD reference checkout exists (default /root/reference, or
$HODLRND_REFERENCE):

    python tests/golden/make_golden.py

For every case in tests/cases.py::REF_CASES it compiles the reference's own
headers in place for that case's hyper-parameters (oracle/build.py::build_ref),
runs oracle/ref_driver.cpp on the seeded points and stores what the reference
produced: tree level sizes, node point counts, neighbour and interaction lists,
the leaf point order, each far block's rank and representation, one matvec,
one GMRES solve (x0 = b, restart 100, tol = eps_ACA, as HODLRdD_matrix::solve)
and the print_matrix_statistics figures.

It also stores the reference's golden pair data/x_10000.bin / data/rhs_10000.bin
(kernel_4d_test, numPoints = 10) with the reference's HODLR matvec of that x at
its shipped hyper-parameters, and a dense-operator GMRES run used to pin the
GMRES restatement bit for bit, and the SHA-256 of the two vector files.

    python tests/golden/make_golden.py vecfiles   # only ref_vec_files.json
"""
import hashlib
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import build, refio  # noqa: E402
from oracle.oracle import dense_matvec  # noqa: E402
import cases  # noqa: E402

REF_DATA = os.path.join(build.REF_ROOT, "data")


def run_driver(exe, mode, args):
    subprocess.run([exe, mode] + args, check=True, stdout=subprocess.DEVNULL)


def make_case(name, c, tmp):
    pts = cases.points(c)
    x, b = cases.vectors(c)
    lo, hi = cases.box(c)
    exe = build.build_ref(c["ndim"], c["nmax"], c["dprime"], c["eps"])
    inp, out = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    refio.write_driver_input(inp, pts, lo, hi, c["kind"], c["scale"], c["diag"], x, b, 100, 0, c["eps"])
    run_driver(exe, "hodlr", [inp, out])
    R = refio.read_named_arrays(out)
    y_dense = dense_matvec(pts, x, kind=c["kind"], scale=c["scale"], diag=c["diag"])
    arrays = dict(points=pts, x=x, b=b, y=R["y"], x_solve=R["x_solve"], y_dense_rel_err=[
                      np.linalg.norm(R["y"] - y_dense) / np.linalg.norm(y_dense)],
                  gmres_iters=R["gmres_iters"], gmres_resid=R["gmres_resid"], stats=R["stats"][:2])
    for k in ("level_sizes", "node_counts", "nbr_ptr", "nbr", "intr_ptr", "intr", "leaf_perm",
              "blk_level", "blk_t", "blk_s", "blk_rank", "blk_memeff"):
        arrays[k] = R[k].astype(np.int32)
    np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **arrays)
    print(f"{name}: {len(R['blk_rank'])} blocks, max rank {R['blk_rank'].max()}, "
          f"{int(R['gmres_iters'][0])} GMRES iterations")


def make_golden4d(tmp):
    g = cases.GOLDEN4D
    x = refio.read_cereal_vector(os.path.join(REF_DATA, "x_10000.bin"))
    rhs = refio.read_cereal_vector(os.path.join(REF_DATA, "rhs_10000.bin"))
    exe = build.build_ref(g["ndim"], g["nmax"], g["dprime"], g["eps"], user_kernels=True)
    xr, out = os.path.join(tmp, "x.raw"), os.path.join(tmp, "g4d.bin")
    x.astype("<f8").tofile(xr)
    run_driver(exe, "golden4d", [xr, out])
    R = refio.read_named_arrays(out)
    np.savez_compressed(os.path.join(HERE, "golden_kernel4d_n10000.npz"), x=x, rhs=rhs,
                        ref_hodlr=R["hodlr"], ref_kii=R["kii"])
    print("golden4d: dense vs rhs", np.linalg.norm(R["dense"] - rhs) / np.linalg.norm(rhs))


def make_vec_files():
    """SHA-256 and size of the reference's own vector files, so that the
    product's save_vec can be checked byte for byte against them."""
    out = {}
    for name in ("x_10000.bin", "rhs_10000.bin"):
        with open(os.path.join(REF_DATA, name), "rb") as f:
            buf = f.read()
        out[name] = {"bytes": len(buf), "sha256": hashlib.sha256(buf).hexdigest()}
    with open(os.path.join(HERE, "ref_vec_files.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("vec files:", out)


def make_dense_gmres(tmp):
    c = dict(ndim=2, n=300, nmax=64, dprime=0, eps=1e-12, kind=cases.INV_R, scale=1.0 / 300,
             diag=1.0, lo=-1.0, hi=1.0, seed=7)
    pts = cases.points(c)
    x, b = cases.vectors(c)
    lo, hi = cases.box(c)
    exe = build.build_ref(c["ndim"], c["nmax"], c["dprime"], c["eps"])
    inp, out = os.path.join(tmp, "in.bin"), os.path.join(tmp, "out.bin")
    # restart 7 exercises the restart path (GMRES.hpp:271-295)
    refio.write_driver_input(inp, pts, lo, hi, c["kind"], c["scale"], c["diag"], x, b, 7, 0, c["eps"])
    run_driver(exe, "gmres", [inp, out])
    R = refio.read_named_arrays(out)
    np.savez_compressed(os.path.join(HERE, "ref_dense_gmres_n300.npz"), points=pts, b=b, restart=7,
                        tol=c["eps"], scale=c["scale"], x_solve=R["x_solve"], gmres_iters=R["gmres_iters"],
                        gmres_resid=R["gmres_resid"])
    print("dense gmres:", int(R["gmres_iters"][0]), "iterations")


def main():
    if not os.path.isdir(build.REF_INCLUDE):
        sys.exit(f"reference checkout not found at {build.REF_ROOT}")
    make_vec_files()
    with tempfile.TemporaryDirectory() as tmp:
        make_golden4d(tmp)
        make_dense_gmres(tmp)
        for name, c in cases.REF_CASES.items():
            make_case(name, c, tmp)


if __name__ == "__main__":
    if sys.argv[1:] == ["vecfiles"]:
        make_vec_files()
    else:
        main()
