#!/usr/bin/env python3
"""HODLR solve throughput on one GB300 (and N independent replicas).

Workload (HODLR3D, mixed precision): NDIM=3, N=262144 points i.i.d. uniform
in [0,1]^3 (numpy PCG64, seeded), A_ij = 1/(N^(2/3) |x_i - x_j|), A_ii = 1,
d' = 0, Nmax = 64, eps_ACA = 1e-8; far-field U, V stored in FP32; solves to a
relative residual of 1e-8; right-hand sides i.i.d. N(0,1).  Three engines:
fp32_factors (headline: FP32 factors with compensated FP32 accumulation inside
FP64 GMRES), mixed (FP64 iterative refinement around FP32 GMRES) and fp64.

A step is one solve on the device-resident operator (the reference's
HODLRdD_matrix::solve, include/HDD_matrix.hpp:51-62), with its right-hand side
already in HBM; the operator build (tree, ACA, leaf blocks) happens once
before the timed region and is reported separately.  `e2e` repeats the steps
through the host-pointer C ABI call (hodlr_solve), the copies in and out of
pinned host memory inside the timed region.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

With N > 1 (torchrun) every rank builds and solves its own instance
(different seed): replicas, no collective on the data path.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_POINTS = 262144
NDIM, NMAX, DPRIME, EPS = 3, 64, 0, 1e-8
SEED = 20261203
METRIC = "solves/s (mixed FP32/FP64 HODLR3D solve to 1e-8 rel. residual)"
MATVEC_REPS = 10
DENSE_ROWS = 2048
SERVING_MAX_ITER = 400


def max_over_ranks(value, world, device="cuda"):
    """The largest value over the ranks: the job's time is its slowest
    replica's (one all-reduce of a scalar, after the timed region)."""
    if world <= 1:
        return value
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def job_rate(steps, world, seconds):
    """Whole-job throughput: every rank's steps over the slowest rank's time."""
    return steps * world / seconds


def workload(n, rank):
    rng = np.random.default_rng(SEED + rank)
    pts = rng.uniform(0.0, 1.0, (n, NDIM))
    return pts, 1.0 / n ** (2.0 / 3.0)


def config(n, impl_note):
    return {"workload": f"HODLR3D solve, N={n} uniform [0,1]^3, A_ij=1/(N^(2/3) r), A_ii=1, d'=0, Nmax=64, "
                        f"eps_ACA=1e-8, FP32-stored far-field factors, solve to 1e-8 rel. residual",
            "n": n, "ndim": NDIM, "nmax": NMAX, "dprime": DPRIME, "eps_aca": EPS, "tol": EPS, "restart": 100,
            "rhs": "N(0,1), one per step", "l2": "inputs larger than L2 (the stored operator is several GB)",
            "impl_note": impl_note}


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi samples (every 200 ms) of this GPU while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id):
        self.gpu_id = gpu_id
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu_id), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def traffic_from_profiles(kernel):
    """DRAM bytes per launch of `kernel` recorded from an ncu capture (profiles/ncu_traffic.txt)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    try:
        for ln in open(path):
            parts = ln.split()
            if len(parts) >= 2 and parts[0] == kernel and not ln.startswith("#"):
                return float(parts[1])
    except OSError:
        pass
    return None


def build_oracle(pts, scale):
    """The CPU oracle (the reference algorithm restated in C++, OpenMP over all
    host cores) built on the workload's points; (oracle, build seconds)."""
    from oracle.oracle import OracleHODLR

    t0 = time.perf_counter()
    O = OracleHODLR(pts, [0.0] * NDIM, [1.0] * NDIM, nmax=NMAX, dprime=DPRIME, eps=EPS, kind=1, scale=scale,
                    diag=1.0, rng_mode=1, threads=os.cpu_count() or 1)
    return O, time.perf_counter() - t0


def cpu_baseline(O, t_build, b):
    """One full FP64 solve by the CPU oracle (x0 = b, restart 100, tol 1e-8),
    timed on all host cores: a measured solve, not an extrapolation."""
    cores = os.cpu_count() or 1
    t0 = time.perf_counter()
    _, iters, res = O.solve(b, restart=100, tol=EPS)
    solve_s = time.perf_counter() - t0
    return {"value": round(1.0 / solve_s, 5), "unit": "solves/s", "cores": cores, "kind": "port",
            "sample": f"one full FP64 solve by the CPU oracle (reference algorithm restated in C++, OpenMP) on the "
                      f"same N={O.n} operator: {iters} GMRES iterations in {solve_s:.1f} s (rel. residual "
                      f"{res:.1e}); build {t_build:.1f} s not included"}


def parity_at_size(O, M64, pts, scale, x_sol, b_sol, stream):
    """Accuracy of the benchmark configuration at its own size: (i) the GPU
    FP64 matvec of a random x against the oracle's HODLR matvec of the same x
    (both the reference algorithm, same ranks); (ii) sampled rows of the direct
    N^2 kernel: the FP64 HODLR matvec's error and the headline solution's
    residual against the dense operator, on DENSE_ROWS rows drawn at random."""
    import torch

    from oracle.oracle import dense_matvec

    n = len(pts)
    rng = np.random.default_rng(SEED + 77)
    x = rng.standard_normal(n)
    y_gpu = M64 * x
    y_orc = O.matvec(x)
    rows = np.sort(rng.choice(n, DENSE_ROWS, replace=False))
    kw = dict(kind=1, scale=scale, diag=1.0, rows=rows)
    yd = dense_matvec(pts, x, **kw)
    ax = dense_matvec(pts, x_sol, **kw)
    bs = b_sol[rows]
    return {"gpu_fp64_matvec_vs_oracle_matvec": float(np.linalg.norm(y_gpu - y_orc) / np.linalg.norm(y_orc)),
            "dense_rows": DENSE_ROWS,
            "gpu_fp64_matvec_vs_dense_rows": float(np.linalg.norm(y_gpu[rows] - yd) / np.linalg.norm(yd)),
            "oracle_matvec_vs_dense_rows": float(np.linalg.norm(y_orc[rows] - yd) / np.linalg.norm(yd)),
            "solution_residual_dense_rows": float(np.linalg.norm(bs - ax) / np.linalg.norm(bs))}


def timed_solves(M, B, X, ks, stream):
    """Solves of right-hand sides B[k], k in ks, into X[k % len(X)] on the
    device; (total ms, per-step ms, infos)."""
    import torch

    sp = stream.cuda_stream
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in ks]
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    infos = []
    torch.cuda.synchronize()
    t0.record(stream)
    for (a, b), k in zip(ev, ks):
        a.record(stream)
        infos.append(M.solve_device(B[k].data_ptr(), X[k % X.shape[0]].data_ptr(), 1, sp))
        b.record(stream)
    t1.record(stream)
    torch.cuda.synchronize()
    return t0.elapsed_time(t1), np.array([a.elapsed_time(b) for a, b in ev]), infos


def matvec_rate(M, x, y, stream):
    """Single-RHS operator application y = A x on device vectors: ms per matvec
    and the algorithmic HBM bytes of one application (the traced kernels' bytes:
    every factor and leaf entry once, the vectors once per reader) over that time."""
    import torch

    sp = stream.cuda_stream
    for _ in range(3):
        M.matvec_device(x.data_ptr(), y.data_ptr(), 1, sp)
    M.trace(True)
    t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record(stream)
    for _ in range(MATVEC_REPS):
        M.matvec_device(x.data_ptr(), y.data_ptr(), 1, sp)
    t1.record(stream)
    torch.cuda.synchronize()
    tr = M.trace()
    M.trace(False)
    ms = t0.elapsed_time(t1) / MATVEC_REPS
    nbytes = sum(v["bytes_per_launch"] * v["launches"] for v in tr.values()) / MATVEC_REPS
    groups = {k: {"ms": round(v["total_ms"] / v["launches"], 4),
                  "GBps": round(v["bytes_per_launch"] / (v["total_ms"] / v["launches"] / 1e3) / 1e9, 1)}
              for k, v in tr.items() if v["launches"]}
    return {"ms": round(ms, 4), "bytes": nbytes, "GBps": round(nbytes / (ms / 1e3) / 1e9, 1), "groups": groups}


def run_gb300(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import hodlrnd_gb300 as h
    from hodlrnd_gb300 import _lib

    n = args.n
    pts, scale = workload(n, rank)
    kern = h.Kernel("inv_r", scale, 1.0)
    box = ([0.0] * NDIM, [1.0] * NDIM)
    common = dict(Nmax=NMAX, eps_ACA=EPS, INTERACTION_TYPE_ALLOWED=DPRIME, tol=EPS, device=local,
                  fp64_check=not args.no_fp64_check)
    t0 = time.perf_counter()
    M = h.HODLRdD_matrix(kern, pts, *box, precision=args.precision, **common).Assemble_matrix_operators()
    build_s = time.perf_counter() - t0
    stats = M.statistics()
    others = {}
    if not args.headline_only:
        for prec in ("fp64", "mixed", "fp32_factors", "bf16_factors"):
            if prec != args.precision:
                others[prec] = h.HODLRdD_matrix(kern, pts, *box, precision=prec, **common).Assemble_matrix_operators()

    K, W = args.steps, args.warmup
    g = torch.Generator(device="cuda").manual_seed(SEED + 1000 + rank)
    B = torch.randn((K + W, n), generator=g, dtype=torch.float64, device="cuda")
    X = torch.empty_like(B)
    stream = torch.cuda.current_stream()
    timed_solves(M, B, X, range(K, K + W), stream)  # warm-up

    # ---- timed region: K solves, right-hand sides resident in HBM
    try:
        gpu_id = "GPU-" + str(torch.cuda.get_device_properties(local).uuid)
    except Exception:
        gpu_id = local
    clocks = ClockSampler(gpu_id)
    M.trace(True)
    launches0 = _lib.lib().hodlr_kernel_launches()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks.start()
    total_ms, step_ms, infos = timed_solves(M, B, X, range(K), stream)
    if world > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    launches = _lib.lib().hodlr_kernel_launches() - launches0
    trace = M.trace()
    M.trace(False)
    total_ms = max_over_ranks(total_ms, world)
    value = job_rate(K, world, total_ms / 1e3)

    # ---- the other engines on the same right-hand sides
    k2 = max(1, min(args.other_steps, K))
    engines = {}
    X2 = torch.empty_like(B[:k2])
    for prec, Mo in others.items():
        timed_solves(Mo, B, X2, [K], stream)
        ms, _, inf = timed_solves(Mo, B, X2, range(k2), stream)
        engines[prec] = {"value": round(k2 / (ms / 1e3), 3), "unit": "solves/s", "steps": k2,
                         "inner_iterations": [i["iterations"] for i in inf],
                         "outer_iterations": [i["outer_iterations"] for i in inf],
                         "rel_residual": max(i["rel_residual"] for i in inf),
                         "rel_residual_stored_operator": max(i["rel_residual_stored"] for i in inf)}
        if "fp64" in others and prec != "fp64":
            b0 = B[0].cpu().numpy()
            engines[prec]["rel_residual_fp64_operator"] = float(
                np.linalg.norm(b0 - others["fp64"] * X2[0].cpu().numpy()) / np.linalg.norm(b0))

    # ---- single-RHS matvec throughput of each engine's operator: compensated
    # products, and for FP32 and BF16 factors also the relaxed (plain FP32)
    # products the solver's inner iterations use
    ops_by_prec = dict([(args.precision, M)] + list(others.items()))
    matvec = {p: matvec_rate(Mm, B[0], X2[0], stream) for p, Mm in ops_by_prec.items()}
    for p in ("fp32_factors", "bf16_factors"):
        if p in ops_by_prec:
            ops_by_prec[p].set_relax("always")
            matvec[p]["relaxed"] = matvec_rate(ops_by_prec[p], B[0], X2[0], stream)
            ops_by_prec[p].set_relax(True)
    if "fp32_factors" in matvec and "bf16_factors" in matvec:
        f, b = matvec["fp32_factors"], matvec["bf16_factors"]
        matvec["bf16_over_fp32_ms"] = {"compensated": round(b["ms"] / f["ms"], 3),
                                       "relaxed": round(b["relaxed"]["ms"] / f["relaxed"]["ms"], 3)}

    # ---- accuracy of the headline solution against the FP64 operator
    acc = {}
    if "fp64" in others:
        M64 = others["fp64"]
        x0, b0 = X[0].cpu().numpy(), B[0].cpu().numpy()
        acc["rel_residual_fp64_operator"] = float(np.linalg.norm(b0 - M64 * x0) / np.linalg.norm(b0))
        x64 = torch.empty_like(B[:1])
        M64.solve_device(B[0].data_ptr(), x64[0].data_ptr(), 1, stream.cuda_stream)
        torch.cuda.synchronize()
        x64 = x64[0].cpu().numpy()
        acc["rel_diff_vs_fp64_solution"] = float(np.linalg.norm(x0 - x64) / np.linalg.norm(x64))
        # a known solution (the reference's self-check, include/main.cpp:42-57): b = A64 x_true,
        # solved by the headline engine and by the FP64 engine; both errors are bounded by the
        # conditioning times the 1e-8 residual, so the headline's is compared with the FP64 engine's
        x_true = np.random.default_rng(SEED + 99).standard_normal(n)
        b_true = M64 * x_true
        x_h, x_f = M.solve(b_true), M64.solve(b_true)
        acc["known_solution"] = {
            "rel_error_headline": float(np.linalg.norm(x_h - x_true) / np.linalg.norm(x_true)),
            "rel_error_fp64_engine": float(np.linalg.norm(x_f - x_true) / np.linalg.norm(x_true)),
            "rel_residual_headline_fp64_operator": float(np.linalg.norm(b_true - M64 * x_h) / np.linalg.norm(b_true)),
            "rel_residual_fp64_engine": float(np.linalg.norm(b_true - M64 * x_f) / np.linalg.norm(b_true))}

    # ---- end to end through the host-pointer C ABI (pinned host buffers)
    hb = torch.empty((K, n), dtype=torch.float64, pin_memory=True)
    hx = torch.empty((K, n), dtype=torch.float64, pin_memory=True)
    hb.copy_(B[:K].cpu())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for k in range(K):
        M.solve(hb[k].numpy(), out=hx[k].numpy())
    e2e_s = time.perf_counter() - t0
    e2e_s = max_over_ranks(e2e_s, world)

    # ---- roofline of the dominant kernel (largest share of traced device time)
    dom = max(trace.items(), key=lambda kv: kv[1]["total_ms"]) if trace else None
    peak, peak_src = measured_hbm_peak()
    roofline = None
    if dom:
        name, d = dom
        per_launch_s = d["total_ms"] / d["launches"] / 1e3
        achieved = d["bytes_per_launch"] / per_launch_s / 1e9
        roofline = {"bound": "hbm", "kernel": name, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                    "frac": round(achieved / peak, 4), "peak_source": peak_src,
                    "bytes_per_launch": d["bytes_per_launch"], "launches": d["launches"],
                    "avg_launch_us": round(per_launch_s * 1e6, 2),
                    "share_of_traced_ms": round(d["total_ms"] / sum(v["total_ms"] for v in trace.values()), 4),
                    "traffic": traffic_from_profiles(name)}

    out = {"metric": METRIC, "value": round(value, 3),
           "unit": "solves/s", "n_gpus": world, "steps": K, "warmup": W, "ms_per_step": round(total_ms / K, 3),
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp32+fp64",
           "data": "synthetic (seeded uniform points, N(0,1) right-hand sides)",
           "config": config(n, ENGINE_NOTES[args.precision]),
           "latency_ms": {"p50": round(float(np.percentile(step_ms, 50)), 3),
                          "p99": round(float(np.percentile(step_ms, 99)), 3)},
           "solve": dict({"engine": args.precision, "inner_iterations": [i["iterations"] for i in infos],
                          "outer_iterations": [i["outer_iterations"] for i in infos],
                          "rel_residual_engine": max(i["rel_residual"] for i in infos),
                          "rel_residual_stored_operator": max(i["rel_residual_stored"] for i in infos),
                          "stop_tol": infos[0]["stop_tol"], "target_rel_error": EPS,
                          "accuracy_check": "FP64 operator (iterative refinement with the FP64 far field)"}, **acc),
           "engines": engines,
           "matvec": matvec,
           "build": {"s": round(build_s, 3), "tree_s": round(stats["t_tree_s"], 3),
                     "aca_s": round(stats["t_aca_s"], 3), "aca_kernel_s": round(stats["t_aca_kernel_s"], 3),
                     "compact_s": round(stats["t_compact_s"], 3), "aca_entries": stats["aca_entries"],
                     "aca_entries_per_s": round(stats["aca_entries"] / max(stats["t_aca_kernel_s"], 1e-9), 1),
                     "near_s": round(stats["t_near_s"], 3),
                     "far_blocks": stats["n_far_blocks"], "dense_far_blocks": stats["n_dense_far_blocks"],
                     "max_rank": stats["max_rank"], "far_bytes": stats["far_bytes"],
                     "near_bytes": stats["near_bytes"], "device_bytes": stats["device_bytes"],
                     "n_flop_reference_metric": stats["n_flop"]},
           "roofline": roofline,
           "trace": {k: {"launches": v["launches"], "ms": round(v["total_ms"], 3),
                         "GBps": round(v["bytes_per_launch"] * v["launches"] / (v["total_ms"] / 1e3) / 1e9, 1)}
                     for k, v in trace.items()},
           "e2e": {"value": round(job_rate(K, world, e2e_s), 3), "unit": "solves/s", "h2d_bytes_per_step": 8 * n,
                   "d2h_bytes_per_step": 8 * n},
           "gpu_launches": int(launches), "clocks": clk}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        O, t_orc = build_oracle(pts, scale)
        if "fp64" in others:
            out["solve"]["at_size"] = parity_at_size(O, others["fp64"], pts, scale, X[0].cpu().numpy(),
                                                     B[0].cpu().numpy(), stream)
        out["cpu_baseline"] = cpu_baseline(O, t_orc, B[0].cpu().numpy())
        del O
    if rank == 0:
        print(json.dumps(out), flush=True)
    M.close()
    for Mo in others.values():
        Mo.close()
    if world > 1:
        torch.distributed.destroy_process_group()


ENGINE_NOTES = {
    "fp32_factors": "far-field U, V stored in FP32, products accumulated in compensated FP32 (Dot2); FP64 near "
                    "field; FP64 GMRES (restart 100, x0 = b) on the FP32-stored operator",
    "mixed": "far-field U, V in FP32; FP64 iterative refinement around FP32 GMRES (inner tol 1e-4)",
    "fp64": "all FP64 (the reference's arithmetic)",
    "bf16_factors": "far-field U, V and dense far tiles in BF16 with FP32 per-row / per-column scales; FP64 near "
                    "field; FP64 GMRES on the BF16-stored operator (its residual against the FP64 operator is the "
                    "BF16 rounding of the far field, about 1e-3)",
}


def run_reference(args):
    """The reference's algorithm on the host cores: the CPU oracle (a C++
    restatement of HODLRnD's tree, ACA, matvec and GMRES, OpenMP over blocks and
    nodes).  The reference's own headers only build here against a project
    shim (and single-threaded), so the oracle stands in for them.  Each timed
    step is one full FP64 solve (x0 = b, restart 100, tol 1e-8) of a fresh
    N(0,1) right-hand side on the operator built before the timed region;
    warm-up steps are single GMRES iterations (the oracle has nothing to warm)."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    n = args.n
    pts, scale = workload(n, 0)
    cores = os.cpu_count() or 1
    O, t_build = build_oracle(pts, scale)
    rng = np.random.default_rng(SEED + 1000)
    for _ in range(args.warmup):
        O.solve(rng.standard_normal(n), restart=1, max_iter=1, tol=1e-300)
    step_s, iters, worst = [], [], 0.0
    t_all = time.perf_counter()
    for _ in range(args.steps):
        bb = rng.standard_normal(n)
        t0 = time.perf_counter()
        _, it, res = O.solve(bb, restart=100, tol=EPS)
        step_s.append(time.perf_counter() - t0)
        iters.append(it)
        worst = max(worst, res)
    total_s = time.perf_counter() - t_all
    ms = 1e3 * total_s / args.steps
    value = args.steps / total_s
    sample = (f"{args.steps} full FP64 solves of the same N={n} operator by the CPU oracle on {cores} host cores "
              f"({min(iters)}-{max(iters)} GMRES iterations each, worst rel. residual {worst:.1e}); build "
              f"{t_build:.1f} s not timed")
    out = {"impl": "reference", "metric": METRIC,
           "value": round(value, 5), "unit": "solves/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": round(ms, 3), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "fp64", "data": "synthetic (seeded uniform points, N(0,1) right-hand sides)",
           "config": config(n, "CPU oracle: the reference algorithm restated in C++ (FP64 throughout)"),
           "latency_ms": {"p50": round(1e3 * float(np.percentile(step_s, 50)), 3),
                          "p99": round(1e3 * float(np.percentile(step_s, 99)), 3)},
           "cpu_baseline": {"value": round(value, 5), "unit": "solves/s", "cores": cores, "kind": "port",
                            "sample": sample},
           "e2e": {"value": round(value, 5), "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def serving_trace(count, seed, pool):
    """The serving workload: Poisson arrivals (mean 200 requests/s) of solve
    requests on geometries drawn from a pool of `pool` seeded point clouds,
    NDIM in {2, 3}, N log-uniform in [4096, 262144], kernel in {1/r, log r
    (2D only), exp(-r)}, A_ii = 1, off-diagonals scaled by 1/N^((d-1)/d),
    1-16 right-hand sides N(0,1), eps_ACA = tol = 1e-8.  GMRES stops at
    SERVING_MAX_ITER iterations: with the 1/sqrt(N) scaling, 2D 1/r systems
    stagnate under GMRES(100); such requests count as not converged."""
    rng = np.random.default_rng(seed)
    geos = []
    for g in range(pool):
        d = int(rng.choice([2, 3]))
        n = int(round(np.exp(rng.uniform(np.log(4096), np.log(262144)))))
        kinds = ["inv_r", "exp_neg_r"] + (["log_r"] if d == 2 else [])
        kind = str(rng.choice(kinds))
        geos.append(dict(d=d, n=n, kind=kind, seed=int(rng.integers(1 << 30)), key=g + 1))
    t = 0.0
    reqs = []
    for i in range(count):
        t += rng.exponential(1.0 / 200.0)
        g = geos[int(rng.integers(pool))]
        reqs.append(dict(t=t, geo=g, nrhs=int(rng.integers(1, 17)), seed=int(rng.integers(1 << 30))))
    return reqs


def run_serving(args):
    """Replays the serving trace twice on one GPU: through the request loop
    (FP32 factors, concurrent slots, resident geometries, admission under a
    150 GiB budget) and as the plain FP64 path (one request at a time, each
    geometry built for its request).  Latency = submit -> solution on the host."""
    import hodlrnd_gb300 as h
    from hodlrnd_gb300.server import Server

    reqs = serving_trace(args.requests, SEED + 5, args.pool)
    pts_cache = {}

    def points(g):
        if g["key"] not in pts_cache:
            pts_cache[g["key"]] = np.random.default_rng(g["seed"]).uniform(0.0, 1.0, (g["n"], g["d"]))
        return pts_cache[g["key"]]

    def kernel(g):
        return h.Kernel(g["kind"], 1.0 / g["n"] ** ((g["d"] - 1) / g["d"]), 1.0)

    def rhs(r):
        return np.random.default_rng(r["seed"]).standard_normal((r["geo"]["n"], r["nrhs"]))

    for r in reqs:  # inputs prepared before the clock starts
        points(r["geo"])
        r["b"] = rhs(r)

    def replay(slots, precision, resident):
        srv = Server(slots=slots, memory_budget_bytes=150 << 30)
        tickets = []
        t0 = time.perf_counter()
        for r in reqs:
            delay = t0 + r["t"] - time.perf_counter()
            if delay > 0:
                time.sleep(delay)
            g = r["geo"]
            box = ([0.0] * g["d"], [1.0] * g["d"])
            key = g["key"] if resident else 0
            tickets.append(srv.submit(points(g), r["b"], kernel(g), box=box, key=key, ndim=g["d"], Nmax=64,
                                      eps_ACA=EPS, tol=EPS, precision=precision, max_iter=SERVING_MAX_ITER))
        lat, res, worst, failed = [], [], 0.0, []
        for r, tk in zip(reqs, tickets):
            x, info = srv.wait(tk)
            lat.append(info["t_total_s"])
            res.append(info)
            if info["status"] == 0:
                worst = max(worst, info["rel_residual"])
            else:
                failed.append(r)
        wall = time.perf_counter() - t0
        st = srv.stats()
        srv.close()
        nrhs = sum(r["nrhs"] for r in reqs)
        ok = [i for i in res if i["status"] == 0]
        ok_rhs = sum(r["nrhs"] for r, i in zip(reqs, res) if i["status"] == 0)
        lat_ok = [i["t_total_s"] for i in ok]
        # the fraction of the replay's device time during which two or more requests ran
        iv = sorted((i["t_device_start_s"], i["t_device_end_s"]) for i in res if i["t_device_end_s"] > 0)
        edges = sorted([(a, 1) for a, _ in iv] + [(b, -1) for _, b in iv])
        busy = multi = 0.0
        level, last = 0, None
        for t, dlt in edges:
            if last is not None and level > 0:
                busy += t - last
                if level > 1:
                    multi += t - last
            level += dlt
            last = t
        out = {"solves_per_s": round(nrhs / wall, 3), "requests_per_s": round(len(reqs) / wall, 3),
               "p50_ms": round(1e3 * float(np.percentile(lat, 50)), 2),
               "p99_ms": round(1e3 * float(np.percentile(lat, 99)), 2), "wall_s": round(wall, 3),
               "converged_requests": len(ok), "converged_solves_per_s": round(ok_rhs / wall, 3),
               "converged_p50_ms": round(1e3 * float(np.percentile(lat_ok, 50)), 2) if lat_ok else None,
               "converged_p99_ms": round(1e3 * float(np.percentile(lat_ok, 99)), 2) if lat_ok else None,
               "worst_rel_residual_converged": worst, "not_converged_requests": len(failed),
               "builds": st["builds"], "resident_hits": st["resident_hits"], "evictions": st["evictions"],
               "device_time_with_overlap": round(multi / busy, 3) if busy > 0 else 0.0,
               "prediction_over_actual": round(float(np.median([i["predicted_bytes"] / i["actual_bytes"]
                                                                 for i in res if i["built"] and i["actual_bytes"]])),
                                               3)}
        return out, failed

    served, failed = replay(args.slots, "fp32_factors", True)
    plain, _ = replay(1, "fp64", False)
    # parity of the failures: the CPU oracle (the reference algorithm, FP64,
    # GMRES(100), the same iteration cap) on the smallest requests that did not
    # converge -- the reference stagnates on them too
    from oracle.oracle import OracleHODLR

    kinds = {"inv_r": 1, "log_r": 3, "exp_neg_r": 4}
    checked = []
    for r in sorted(failed, key=lambda r: r["geo"]["n"])[:args.failed_checks]:
        g = r["geo"]
        k = kernel(g)
        O = OracleHODLR(points(g), [0.0] * g["d"], [1.0] * g["d"], nmax=64, dprime=0, eps=EPS, kind=kinds[g["kind"]],
                        scale=k.scale, diag=1.0, rng_mode=1)
        _, it, res = O.solve(r["b"][:, 0], restart=100, max_iter=SERVING_MAX_ITER, tol=EPS)
        checked.append({"ndim": g["d"], "n": g["n"], "kernel": g["kind"], "oracle_iterations": it,
                        "oracle_rel_residual": res})
        del O
    served["not_converged_checked_with_oracle"] = checked
    out = {"metric": "served solves/s and p50/p99 latency (serving trace)", "value": served["solves_per_s"],
           "unit": "solves/s", "n_gpus": 1, "higher_is_better": True, "dtype": "fp32+fp64", "data": "synthetic",
           "config": {"workload": f"serving trace: {len(reqs)} requests, Poisson arrivals at 200/s, {args.pool} "
                                  "geometries (NDIM 2-3, N log-uniform 4096-262144, 1/r, log r, exp(-r)), 1-16 RHS, "
                                  "tol 1e-8, budget 150 GiB",
                      "slots": args.slots},
           "served": served, "plain_fp64_one_at_a_time": plain}
    print(json.dumps(out), flush=True)


def run_batch(args):
    """The batching workload: args.instances independent 3D operators, N
    log-uniform in [2048, 65536], seeded uniform points in [0,1]^3, A_ij =
    1/(N^(2/3) r), A_ii = 1, d' = 0, Nmax = 64, eps_ACA = 1e-6, FP32 factors
    and vectors; 32 right-hand sides N(0,1) per instance.  Times the batched
    build (shared ACA launches) against building the instances one by one, and
    the batch matvec of all instances and right-hand sides (one CUDA graph)
    against the instances' own matvecs."""
    import torch

    import hodlrnd_gb300 as h
    from hodlrnd_gb300.batch import HODLRdD_batch

    rng = np.random.default_rng(SEED + 3)
    ns = [int(round(np.exp(rng.uniform(np.log(2048), np.log(65536))))) for _ in range(args.instances)]
    pts = [rng.uniform(0.0, 1.0, (n, 3)) for n in ns]
    kern = [h.Kernel("inv_r", 1.0 / n ** (2.0 / 3.0), 1.0) for n in ns]
    box = ([0.0] * 3, [1.0] * 3)
    # matvecs only: no FP64 copy of the far field for refined solves (it would
    # triple the 256 instances' factor memory)
    params = dict(Nmax=64, eps_ACA=1e-6, tol=1e-6, precision="mixed", fp64_check=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    B = HODLRdD_batch(kern, pts, [box] * len(ns), **params)
    t_batch = time.perf_counter() - t0
    t0 = time.perf_counter()
    sample = list(range(0, len(ns), max(1, len(ns) // 16)))  # one-by-one builds of a sample, scaled
    alone = []
    for i in sample:
        alone.append(h.HODLRdD_matrix(kern[i], pts[i], *box, **params).Assemble_matrix_operators())
    t_alone = (time.perf_counter() - t0) * len(ns) / len(sample)
    nrhs = 32
    off = B.offsets
    X = torch.randn((nrhs, int(off[-1])), dtype=torch.float32, device="cuda",
                    generator=torch.Generator(device="cuda").manual_seed(SEED + 4))
    Y = torch.empty_like(X)
    st = torch.cuda.current_stream()
    for _ in range(args.warmup):
        B.matvec_device(X.data_ptr(), Y.data_ptr(), nrhs, st.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(args.steps):
        B.matvec_device(X.data_ptr(), Y.data_ptr(), nrhs, st.cuda_stream)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    # bytes of one single-RHS batch matvec: every instance's factors and near tiles (FP32) once
    from hodlrnd_gb300 import _lib
    import ctypes

    tot_bytes = 0
    for i in range(len(ns)):
        sv = _lib.HodlrStats()
        _lib.check(_lib.lib().hodlr_stats_get(B.op(i), ctypes.byref(sv)))
        tot_bytes += sv.far_bytes + sv.near_bytes // 3  # the FP32 near copy is a third of near_bytes
    # instances' own matvecs (FP64 vectors) of the sample, per right-hand side
    x1 = torch.randn(int(max(ns)), dtype=torch.float64, device="cuda")
    y1 = torch.empty_like(x1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for M in alone:
        for _ in range(4):
            M.matvec_device(x1.data_ptr(), y1.data_ptr(), 1, st.cuda_stream)
    torch.cuda.synchronize()
    t_one = (time.perf_counter() - t0) / 4 * len(ns) / len(sample)
    for M in alone:
        M.close()
    out = {"metric": "batched matvecs/s (instances x right-hand sides)", "value": round(len(ns) * nrhs / (ms / 1e3), 1),
           "unit": "instance-matvecs/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": round(ms, 3), "higher_is_better": True, "dtype": "fp32", "data": "synthetic",
           "config": {"workload": f"{len(ns)} 3D instances, N log-uniform 2048-65536 (total {int(off[-1])}), "
                                  "1/(N^(2/3) r), eps_ACA 1e-6, FP32 factors and vectors, 32 RHS each",
                      "instances": len(ns), "total_points": int(off[-1])},
           "graph_step": "one CUDA graph: every instance and right-hand side, one launch per phase per column",
           # single-RHS-equivalent bytes (every factor byte once per right-hand side) over the step's
           # time: it exceeds the HBM bandwidth because each staged byte serves 32 right-hand sides
           "single_rhs_equivalent_GBps": round(tot_bytes * nrhs / (ms / 1e3) / 1e9, 1),
           "factor_GBps": round(tot_bytes * (nrhs / 32) / (ms / 1e3) / 1e9, 1),
           "build": {"batched_s": round(t_batch, 3), "one_by_one_s_estimated": round(t_alone, 3),
                     "one_by_one_sample": len(sample)},
           "one_by_one_fp64_matvec_s_per_rhs_all_instances": round(t_one, 4),
           "batched_s_per_rhs_all_instances": round(ms / 1e3 / nrhs, 5)}
    print(json.dumps(out), flush=True)
    B.close()


def run_c4(args):
    """The 4D workload: N = 65536 points uniform in [0,1]^4, A_ij =
    1/(N^(1/2) |x_i - x_j|^2), A_ii = 1, Nmax = 128, for d' = -1 and d' = 0:
    eps_ACA = 1e-4 with BF16 per-column-scaled factors and FP32 accumulation,
    then eps_ACA = 1e-8 with FP32 factors (and the FP64 operator beside it);
    for each the build and single right-hand-side matvecs, and a
    64-right-hand-side matvec of the 1e-8 FP32 operator (multi-RHS kernels,
    FP32 vectors, one CUDA graph).  Each reduced-precision product is compared
    with the FP64 operator's on the same x.  With this scaling the operator's
    off-diagonal row sums grow like N^(1/2) and restarted GMRES stagnates
    (relative residual about 0.2 after 600 iterations at N = 8192 in the CPU
    oracle), so the workload is timed on matvecs, not solves."""
    import torch

    import hodlrnd_gb300 as h
    from hodlrnd_gb300.batch import HODLRdD_batch

    n, d = args.n if args.n != N_POINTS else 65536, 4
    rng = np.random.default_rng(SEED + 4)
    pts = rng.uniform(0.0, 1.0, (n, d))
    kern = h.Kernel("inv_r2", 1.0 / n ** 0.5, 1.0)
    box = ([0.0] * d, [1.0] * d)
    st = torch.cuda.current_stream()
    out = {"metric": "4D single-RHS and 64-RHS matvecs/s", "unit": "matvecs/s", "n_gpus": 1, "higher_is_better": True,
           "data": "synthetic", "dtype": "bf16+fp32+fp64",
           "config": {"workload": f"4D, N={n} uniform [0,1]^4, 1/(N^(1/2) r^2), A_ii=1, Nmax=128; d' = -1 and 0; "
                                  "eps_ACA=1e-4 BF16 per-column-scaled factors, FP32 accumulation; eps_ACA=1e-8 "
                                  "FP32 factors; 1 and 64 RHS"}, "cases": {}}
    x = torch.randn(n, dtype=torch.float64, device="cuda", generator=torch.Generator(device="cuda").manual_seed(SEED))
    y = torch.empty_like(x)
    X = torch.randn((64, n), dtype=torch.float32, device="cuda", generator=torch.Generator(device="cuda").manual_seed(SEED))
    x0 = X[0].to(torch.float64)  # column 0 of the 64-RHS inputs, for single-RHS comparisons
    reps = max(args.steps, 3)
    engines = (("bf16_factors", 1e-4, "always"), ("fp32_factors", 1e-8, True), ("fp64", 1e-8, True))
    if args.c4_engine != "all":  # one engine alone (a small case for profiling)
        engines = tuple(e for e in engines if e[0] == args.c4_engine)
    for dp in ((-1, 0) if args.c4_dprime is None else (args.c4_dprime,)):
        res, ys = {}, {}
        for prec, eps, relax in engines:
            t0 = time.perf_counter()
            M = h.HODLRdD_matrix(kern, pts, *box, Nmax=128, eps_ACA=eps, INTERACTION_TYPE_ALLOWED=dp,
                                 precision=prec, relax=relax).Assemble_matrix_operators()
            t_build = time.perf_counter() - t0
            r = matvec_rate(M, x, y, st)
            ys[prec] = y.cpu().numpy().copy()
            M.matvec_device(x0.data_ptr(), y.data_ptr(), 1, st.cuda_stream)
            ys[prec + "_x0"] = y.cpu().numpy().copy()
            tc = None
            if prec == "bf16_factors":
                # 64 right-hand sides on the tensor cores (tcgen05, BF16 operands, FP32 accumulation)
                Y = torch.empty_like(X)
                for _ in range(3):
                    M.matvec_tc_device(X.data_ptr(), Y.data_ptr(), 64, st.cuda_stream)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                torch.cuda.synchronize()
                e0.record(st)
                for _ in range(reps):
                    M.matvec_tc_device(X.data_ptr(), Y.data_ptr(), 64, st.cuda_stream)
                e1.record(st)
                torch.cuda.synchronize()
                tms = e0.elapsed_time(e1) / reps
                ys["tc_x0"] = Y[0].double().cpu().numpy().copy()
                tc = {"ms": round(tms, 3), "rhs_matvecs_per_s": round(64 / (tms / 1e3), 1),
                      "operands": "BF16 factors as stored, right-hand sides split into BF16 high and low parts, "
                                  "FP64 near field in three BF16 terms; FP32 accumulation in tensor memory"}
            s = M.statistics()
            res[prec] = {"eps_ACA": eps, "accumulation": "fp32" if relax == "always" else
                         ("fp64" if prec == "fp64" else "compensated fp32"),
                         "matvec_ms": r["ms"], "matvec_GBps": r["GBps"], "matvec_groups": r["groups"],
                         "build_s": round(t_build, 3),
                         "far_blocks": s["n_far_blocks"], "dense_far_blocks": s["n_dense_far_blocks"],
                         "max_rank": s["max_rank"], "far_bytes": s["far_bytes"], "near_bytes": s["near_bytes"],
                         "device_bytes": s["device_bytes"]}
            if tc is not None:
                res[prec]["rhs64_tensor_cores"] = tc
            M.close()
        if args.c4_engine != "all":
            out["cases"][f"dprime={dp}"] = res
            continue
        y64 = ys["fp64"]
        for prec in ("bf16_factors", "fp32_factors"):
            res[prec]["rel_diff_vs_fp64_operator"] = float(np.linalg.norm(ys[prec] - y64) / np.linalg.norm(y64))
        if "tc_x0" in ys:
            t0v, b0v, f0v = ys["tc_x0"], ys["bf16_factors_x0"], ys["fp64_x0"]
            tcr = res["bf16_factors"]["rhs64_tensor_cores"]
            tcr["rel_diff_vs_fp64_operator"] = float(np.linalg.norm(t0v - f0v) / np.linalg.norm(f0v))
            tcr["single_rhs_bf16_rel_diff_vs_fp64_operator"] = float(np.linalg.norm(b0v - f0v) / np.linalg.norm(f0v))
            tcr["rel_diff_vs_single_rhs_bf16"] = float(np.linalg.norm(t0v - b0v) / np.linalg.norm(b0v))
        B = HODLRdD_batch([kern], [pts], [box], Nmax=128, eps_ACA=1e-8, INTERACTION_TYPE_ALLOWED=dp,
                          precision="mixed", fp64_check=False)
        Y = torch.empty_like(X)
        for _ in range(3):
            B.matvec_device(X.data_ptr(), Y.data_ptr(), 64, st.cuda_stream)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        for _ in range(reps):
            B.matvec_device(X.data_ptr(), Y.data_ptr(), 64, st.cuda_stream)
        e1.record(st)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / reps
        res["rhs64_matvec"] = {"ms": round(ms, 3), "rhs_matvecs_per_s": round(64 / (ms / 1e3), 1),
                               "single_rhs_equivalent_speedup_vs_fp32_factors": round(
                                   res["fp32_factors"]["matvec_ms"] * 64 / ms, 2)}
        B.close()
        out["cases"][f"dprime={dp}"] = res
    last = out["cases"][f"dprime={dp}"]
    out["value"] = (last["rhs64_matvec"]["rhs_matvecs_per_s"] if "rhs64_matvec" in last
                    else round(1e3 / next(iter(last.values()))["matvec_ms"], 1))
    print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--n", type=int, default=N_POINTS)
    ap.add_argument("--precision", choices=["fp32_factors", "mixed", "fp64", "bf16_factors"],
                    default="fp32_factors", help="engine timed for `value`; the others are timed beside it")
    ap.add_argument("--other-steps", type=int, default=3)
    ap.add_argument("--headline-only", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-check", action="store_true",
                    help="reduced-precision engines without the FP64 far field (stop on the stored operator)")
    ap.add_argument("--instances", type=int, default=256)
    ap.add_argument("--workload", choices=["solve", "serving", "batch", "c4"], default="solve",
                    help="serving: replay the request trace through the request loop (its own JSON line)")
    ap.add_argument("--requests", type=int, default=48)
    ap.add_argument("--c4-engine", choices=["all", "bf16_factors", "fp32_factors", "fp64"], default="all",
                    help="c4: time one engine alone (no 64-RHS pass, no comparison)")
    ap.add_argument("--c4-dprime", type=int, choices=[-1, 0], default=None, help="c4: one d' only")
    ap.add_argument("--pool", type=int, default=12)
    ap.add_argument("--slots", type=int, default=4)
    ap.add_argument("--failed-checks", type=int, default=3,
                    help="serving: requests that did not converge re-solved by the CPU oracle")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be at least 3")
    if args.workload == "serving":
        run_serving(args)
    elif args.workload == "batch":
        run_batch(args)
    elif args.workload == "c4":
        run_c4(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_gb300(args)


if __name__ == "__main__":
    main()
