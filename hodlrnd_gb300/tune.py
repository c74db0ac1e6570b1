"""Ring-shape tuner for the staged matvec kernels.

    python -m hodlrnd_gb300.tune [--n 262144] [--solves 4] [--variants JSON]

The staged kernels of csrc/matvec.cu take their ring shapes (stages per warp
and bytes per stage of V^T x, node-panel and leaf-panel rings, and the
leaf/node-panel CTAs per SM the register allocation must allow) from
HODLR_TUNE_* macros, and the plan's item sizes (Z_ITEM_BYTES: V bytes per
V^T x item; SMALL_ITEM_BYTES: factor bytes per leaf-panel item) too.  For
each variant -- a JSON object of macro overrides, e.g. {"P_STAGES": 3,
"P_BYTES": 2048} -- this builds matvec.cu and engine.cu with those values
into a variant library, links them with the other
objects of the in-place build (variant files go to hodlrnd_gb300/_tune/,
git-ignored), and times a headline-engine operator with it
in a child process (HODLRND_LIBRARY selects the library): the build, one
warm-up solve, `--solves` timed solves on device-resident right-hand sides,
and the per-group GB/s of the traced matvec launches.  The variant with the
fewest milliseconds per solve is printed last; its values are the ones to
put in the macros' defaults.  The workload is the bench's (3D, uniform
points, 1/(N^(2/3) r), d' = 0, Nmax = 64, eps_ACA = 1e-8, FP32 factors).

Leaf-panel byte budgets below 2048 are refused by a static_assert in
matvec.cu (a one-row leaf would get no columns per piece).
"""
import argparse
import json
import os
import subprocess
import sys

from . import build as B

DEFAULT_VARIANTS = {
    "default": {},
    "3 stages": {"Z_STAGES": 3, "P_STAGES": 3, "S_STAGES": 3},
    "P 3072 bytes": {"P_BYTES": 3072},
    "Z 3072 bytes": {"Z_BYTES": 3072},
}


# plan-level knobs (item sizes) live in the plan code too, so variants rebuild
# both translation units
TUNED_SOURCES = ("matvec.cu", "engine.cu")


def _variant_lib(name, overrides):
    tdir = os.path.join(B.HERE, "_tune")
    os.makedirs(tdir, exist_ok=True)
    tag = "".join(c if c.isalnum() else "_" for c in name)
    lib = os.path.join(tdir, f"lib_{tag}.so")
    defs = [f"-DHODLR_TUNE_{k}={int(v)}" for k, v in overrides.items()]
    tuned = []
    for src in TUNED_SOURCES:
        obj = os.path.join(tdir, f"{os.path.splitext(src)[0]}_{tag}.o")
        cmd = [B.nvcc(), "-c", os.path.join(B.CSRC, src), "-o", obj, "-std=c++17", "-O3", "-lineinfo",
               "-Xcompiler", B.HOST_FLAGS] + B.ARCH + ["-Xptxas", "-O3"] + defs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"variant {name}: nvcc failed for {src}\n{r.stderr[-2000:]}")
        tuned.append(obj)
    objs = [os.path.join(B.OBJ, os.path.splitext(s)[0] + ".o") for s in B.SOURCES if s not in TUNED_SOURCES]
    r = subprocess.run([B.nvcc(), "-shared", "-o", lib] + tuned + objs + B.ARCH + ["-Xcompiler", "-fopenmp", "-lgomp"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"variant {name}: link failed\n{r.stderr[-2000:]}")
    return lib


def _time_child(n, solves):
    """Runs in the child: times solves of the bench operator with the loaded library."""
    import time

    import numpy as np
    import torch

    import hodlrnd_gb300 as h

    rng = np.random.default_rng(1234)
    pts = rng.uniform(0.0, 1.0, (n, 3))
    M = h.HODLRdD_matrix(h.Kernel("inv_r", 1.0 / n ** (2.0 / 3.0), 1.0), pts, [0.0] * 3, [1.0] * 3,
                         precision="fp32_factors", Nmax=64, eps_ACA=1e-8, INTERACTION_TYPE_ALLOWED=0,
                         tol=1e-8).Assemble_matrix_operators()
    B_ = torch.randn((solves + 1, n), dtype=torch.float64, device="cuda",
                     generator=torch.Generator(device="cuda").manual_seed(5))
    X = torch.empty_like(B_)
    st = torch.cuda.current_stream().cuda_stream
    M.solve_device(B_[solves].data_ptr(), X[solves].data_ptr(), 1, st)
    torch.cuda.synchronize()
    M.trace(True)
    t0 = time.perf_counter()
    its = [M.solve_device(B_[k].data_ptr(), X[k].data_ptr(), 1, st)["iterations"] for k in range(solves)]
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / solves * 1e3
    tr = M.trace()
    groups = {k: round(v["bytes_per_launch"] * v["launches"] / (v["total_ms"] / 1e3) / 1e9, 1)
              for k, v in tr.items() if v["launches"]}
    print(json.dumps({"ms_per_solve": round(ms, 2), "iterations": its, "group_GBps": groups}), flush=True)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--n", type=int, default=262144)
    ap.add_argument("--solves", type=int, default=4)
    ap.add_argument("--variants", type=str, default=None, help="JSON object: name -> {MACRO: value}")
    ap.add_argument("--child", action="store_true", help=argparse.SUPPRESS)
    a = ap.parse_args(argv)
    if a.child:
        _time_child(a.n, a.solves)
        return
    variants = json.loads(a.variants) if a.variants else DEFAULT_VARIANTS
    B.build()
    results = {}
    for name, ov in variants.items():
        lib = _variant_lib(name, ov)
        env = dict(os.environ, HODLRND_LIBRARY=lib)
        r = subprocess.run([sys.executable, "-m", "hodlrnd_gb300.tune", "--child", "--n", str(a.n), "--solves",
                            str(a.solves)], env=env, capture_output=True, text=True,
                           cwd=os.path.dirname(B.HERE))
        if r.returncode != 0:
            print(json.dumps({"variant": name, "overrides": ov, "error": r.stderr[-1000:]}), flush=True)
            continue
        res = json.loads(r.stdout.strip().splitlines()[-1])
        results[name] = res
        print(json.dumps({"variant": name, "overrides": ov, **res}), flush=True)
    if results:
        best = min(results, key=lambda k: results[k]["ms_per_solve"])
        print(json.dumps({"best": best, "overrides": variants[best], **results[best]}), flush=True)


if __name__ == "__main__":
    main()
