#!/usr/bin/env python
"""PCG time to a 1e-8 relative residual on one GB300: FP32-G vs FP64 vs CPU.

Workload: 3D 7-point graph Laplacian on a 256^3 grid (16.8M unknowns) with
edge weights exp(N(0,1)) and diagonal = sum of incident weights + 1e-3
(SDDM), b ~ N(0,1); nested-dissection ordering (METIS, host), randomized
Cholesky factor on the GPU (FP64 accumulation), PCG to 1e-8 verified in FP64.
A "step" is one complete PCG solve.  ``value`` is the FP32-G solve time with
A, G and b resident in HBM; ``e2e`` is the same solve through the C ABI with
host buffers (b copied in, x copied out inside the timed region).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU: the path does not shard (one GPU, no sharding), so N ranks run N
independent replicas; ``value`` is then the time of the slowest replica and
the line reports the aggregate throughput in ``solves_per_s``.

``configs`` adds the other workloads as parity/feature lines: 32 right-hand
sides at 128^3, 512 independent 2D systems in one batched solve, and the
gradient of a 1024^2 solve through the adjoint PCG.
"""

from __future__ import annotations

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

METRIC = "PCG time to 1e-8 residual: FP32-G vs FP64 GPU vs CPU; SpMV/SpTRSV HBM GB/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--n", type=int, default=256, help="grid side")
    p.add_argument("--leaves", type=int, default=0,
                   help="nested-dissection subdomains (0: the tuned count cached for this shape, else 2048)")
    p.add_argument("--tol", type=float, default=1e-8)
    p.add_argument("--maxit", type=int, default=200)
    p.add_argument("--seed", type=int, default=0)
    p.add_argument("--cpu-sample-iters", type=int, default=4)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the k-right-hand-side (128^3, k=32), batched-systems (512 2D grids) and "
                        "differentiation (1024^2 adjoint solve) lines")
    p.add_argument("--config", default="bench", choices=["bench", "c5"],
                   help="c5: the large high-contrast configuration alone (--n 512: 134M unknowns, checkerboard "
                        "of 1 and 1e4 in 8^3-cell blocks, k=8, FP32 G), with device and host peak memory")
    return p.parse_args()


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1 and args.impl == "gb300":
        import torch.distributed as dist

        backend = "nccl" if args.impl == "gb300" else "gloo"
        dist.init_process_group(backend)
        pg = dist
    return rank, local, world, pg


def max_over_ranks(value, pg, device):
    """The slowest replica's time: every rank gets max(value) over ranks."""
    if pg is None:
        return float(value)
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


class SmiSampler:
    """One nvidia-smi query on one GPU every 200 ms, in a background thread,
    while the block runs; `samples` holds (time, fields) pairs."""

    Q = ""

    def __init__(self, gpu_index):
        self.idx = gpu_index
        self.proc = None
        self.samples = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append((time.time(), [x.strip() for x in line.split(",")]))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()


class ClockSampler(SmiSampler):
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, f in self.samples:
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


class MemSampler(SmiSampler):
    """Device memory in use (nvidia-smi, every 200 ms) while the block runs."""

    Q = "memory.used"

    def peak_gb(self, t0=None, t1=None):
        v = []
        for t, f in self.samples:
            if (t0 is None or t >= t0) and (t1 is None or t <= t1):
                try:
                    v.append(float(f[0]))
                except (ValueError, IndexError):
                    pass
        return round(max(v) * 1048576 / 1e9, 2) if v else None


def measured_peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per triangular solve from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "trsv_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


def build_problem(args):
    from rchol_gb300 import generators

    t0 = time.time()
    A = generators.laplace_3d_weighted(args.n, sigma=1.0, shift=1e-3, seed=args.seed)
    b = np.random.default_rng(args.seed + 1).standard_normal(A.shape[0])
    return A, b, time.time() - t0


# --------------------------------------------------------------------------------------
# GB300 arm
# --------------------------------------------------------------------------------------

def run_gb300(args, rank, local, world, pg):
    import torch

    import rchol_gb300 as R
    from rchol_gb300 import _lib

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = _lib.lib()
    A, b, t_gen = build_problem(args)
    n = A.shape[0]
    from rchol_gb300 import tuning

    leaves_source = "argument"
    if args.leaves <= 0:
        args.leaves = tuning.subdomains_for(n, A.nnz, R.PREC_FP32)
        leaves_source = "tuning cache" if tuning.load_cache().get(tuning._key(n, A.nnz, R.PREC_FP32)) else "default"
    t0 = time.time()
    tree = R.Tree.build(A.indptr, A.indices, args.leaves)
    perm, part = tree.arrays()
    t_order = time.time() - t0
    t0 = time.time()
    Ad = R.Matrix.create(A.indptr, A.indices, A.data, tree)
    torch.cuda.synchronize()
    t_upload = time.time() - t0
    t0 = time.time()
    F64 = R.Factor.compute(Ad, tree, seed=args.seed, precision=R.PREC_FP64)
    torch.cuda.synchronize()
    t_factor = time.time() - t0
    setup_split = F64.setup_times()  # factor_gpu = eliminate + assemble + plan (+ the extended Laplacian)
    F32 = R.Factor.compute(Ad, tree, seed=args.seed, precision=R.PREC_FP32)
    knobs32, knobs64 = F32.tune(), F64.tune()  # launch choices timed on each factor
    nnzG = F64.nnz
    nnzA = A.nnz
    bp = np.ascontiguousarray(b[perm])
    d_b = torch.tensor(bp, dtype=torch.float64, device=dev)
    d_x = torch.zeros_like(d_b)
    stream = torch.cuda.current_stream(dev)
    relres = np.zeros(1)
    itr = np.zeros(1, dtype=np.int32)

    def solve(F):
        _lib.check(L.rchol_gpu_pcg_d(Ad.ptr, F.ptr, d_b.data_ptr(), d_x.data_ptr(), 1, args.tol, args.maxit,
                                     _lib.pd(relres), itr.ctypes.data_as(_lib._ip), stream.cuda_stream))
        return float(relres[0]), int(itr[0])

    def barrier():
        if pg is not None:
            pg.barrier()
        torch.cuda.synchronize(dev)

    # RCHOL_PROFILE_TIMED=1 brackets the timed FP32 solves with the CUDA
    # profiler range (cudaProfilerStart/Stop), so that a profiler started with
    # its capture off (ncu --profile-from-start off) sees exactly those launches
    profile_timed = os.environ.get("RCHOL_PROFILE_TIMED") == "1"

    def timed(fn, steps, profile=False):
        for _ in range(args.warmup):
            fn()
        barrier()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        if profile:
            torch.cuda.profiler.start()
        e0.record(stream)
        out = None
        for _ in range(steps):
            out = fn()
        e1.record(stream)
        barrier()
        if profile:
            torch.cuda.profiler.stop()
        ms = max_over_ranks(e0.elapsed_time(e1) / steps, pg, dev)
        return ms, out

    launches0 = L.rchol_gpu_launch_count()
    with ClockSampler(local) as clk:
        ms32, (rr32, it32) = timed(lambda: solve(F32), args.steps, profile=profile_timed)
    launches = (L.rchol_gpu_launch_count() - launches0) // (args.steps + args.warmup)
    x32 = d_x.cpu().numpy()
    ms64, (rr64, it64) = timed(lambda: solve(F64), args.steps)
    x64 = d_x.cpu().numpy()
    # FP64 host verification of both solutions: ||A(p,p) x - b(p)|| / ||b||
    Ap = A[perm][:, perm].tocsr()
    ver32 = float(np.linalg.norm(Ap @ x32 - bp) / np.linalg.norm(bp))
    ver64 = float(np.linalg.norm(Ap @ x64 - bp) / np.linalg.norm(bp))

    # kernel-level rates: one forward triangular solve and one SpMV
    d_y32 = torch.empty_like(d_b)

    def trsv(F):
        _lib.check(L.rchol_gpu_trsv_d(F.ptr, 0, d_b.data_ptr(), d_y32.data_ptr(), 1, stream.cuda_stream))

    def spmv():
        _lib.check(L.rchol_gpu_spmv_d(Ad.ptr, d_b.data_ptr(), d_y32.data_ptr(), 1, stream.cuda_stream))

    trsv32_ms, _ = timed(lambda: trsv(F32), max(3, args.steps))
    trsv64_ms, _ = timed(lambda: trsv(F64), max(3, args.steps))
    spmv_ms, _ = timed(spmv, 20)
    rows = (n + 1) * 8 + 2 * 8 * n  # row pointers + read rhs + write solution
    bytes_trsv32 = nnzG * (4 + 4) + rows
    bytes_trsv64 = nnzG * (8 + 4) + rows
    bytes_spmv = nnzA * (8 + 4) + rows
    peak, peak_kind = measured_peak_hbm()
    gbs = lambda by, ms: by / (ms * 1e-3) / 1e9

    # end to end through the C ABI with host buffers (pinned: b in, x out)
    b_pin = torch.empty(n, dtype=torch.float64, pin_memory=True)
    x_pin = torch.empty(n, dtype=torch.float64, pin_memory=True)
    b_pin.numpy()[:] = bp
    b_host, x_host = b_pin.numpy(), x_pin.numpy()
    rr_h = np.zeros(1)
    it_h = np.zeros(1, dtype=np.int32)

    def solve_host():
        _lib.check(L.rchol_gpu_pcg(Ad.ptr, F32.ptr, _lib.pd(b_host), _lib.pd(x_host), 1, args.tol, args.maxit,
                                   _lib.pd(rr_h), it_h.ctypes.data_as(_lib._ip)))

    for _ in range(args.warmup):
        solve_host()
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        solve_host()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3 / args.steps, pg, dev)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(args, Ap, bp, F64, it64)
    vs_ref = None
    if rank == 0 and not args.no_extras:
        try:
            vs_ref = reference_factor_stats(args, A, perm, part, Ad, tree, bp, nnzG, it64)
        except Exception as exc:  # noqa: BLE001
            vs_ref = {"error": f"{type(exc).__name__}: {exc}"}
    extras = None
    if not args.no_extras:
        del F64, F32, Ad
        extras = {}
        for key, fn in (("k_rhs", run_k_rhs), ("batched", run_batched), ("differentiation", run_differentiation)):
            try:  # a failing extra line is reported in the JSON, the headline stands
                extras[key] = fn(args, dev)
            except Exception as exc:  # noqa: BLE001
                extras[key] = {"error": f"{type(exc).__name__}: {exc}"}
    if rank != 0:
        return None
    traffic = profile_traffic()
    line = {
        "metric": METRIC,
        "value": round(ms32, 3),
        "unit": "ms",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(ms32, 3),
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "fp32-G / fp64-PCG",
        "data": "synthetic (seeded log-normal coefficients, b ~ N(0,1))",
        "config": {
            "workload": f"PCG to {args.tol:g}, 7-point log-normal Laplacian {args.n}^3 (n={n}, nnz(A)={nnzA}), "
                        f"rchol G (nnz={nnzG}) stored and applied in FP32",
            "grid": args.n, "leaves": args.leaves, "leaves_from": leaves_source, "tol": args.tol,
            "tuned_launch": {"fp32": knobs32, "fp64": knobs64},
            "l2": "inputs larger than L2 (A %.2f GB, G %.2f GB)" % (nnzA * 12 / 1e9, nnzG * 8 / 1e9),
            "parallelism": f"replicas x{world}",
        },
        "fp32": {"ms": round(ms32, 3), "iters": it32, "relres_gpu": rr32, "relres_host_fp64": ver32},
        "fp64": {"ms": round(ms64, 3), "iters": it64, "relres_gpu": rr64, "relres_host_fp64": ver64},
        "fp32_speedup_vs_fp64": round(ms64 / ms32, 3),
        "solves_per_s": round(world * 1e3 / ms32, 3),
        "kernels": {
            "trsv_fp32": {"ms": round(trsv32_ms, 4), "GB/s": round(gbs(bytes_trsv32, trsv32_ms), 1)},
            "trsv_fp64": {"ms": round(trsv64_ms, 4), "GB/s": round(gbs(bytes_trsv64, trsv64_ms), 1)},
            "spmv_fp64": {"ms": round(spmv_ms, 4), "GB/s": round(gbs(bytes_spmv, spmv_ms), 1)},
        },
        "roofline": {
            "kernel": "forward triangular solve with G (fp32), all stage launches",
            "bound": "hbm",
            "achieved": round(gbs(bytes_trsv32, trsv32_ms), 1),
            "peak": peak,
            "peak_kind": peak_kind,
            "unit": "GB/s",
            "frac": round(gbs(bytes_trsv32, trsv32_ms) / peak, 4),
            "traffic": (traffic or {}).get("bytes_per_solve"),
        },
        "setup_s": {"generate": round(t_gen, 2), "order": round(t_order, 2), "upload": round(t_upload, 2),
                    "factor_gpu": round(t_factor, 2),
                    **{k: round(v, 2) for k, v in setup_split.items()}},
        "e2e": {"value": round(e2e_ms, 3), "unit": "ms", "h2d_bytes_per_step": 8 * n, "d2h_bytes_per_step": 8 * n},
        "gpu_launches": int(launches),
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "vs_reference_factor": vs_ref,
        "configs": extras,
    }
    return line


def _event_ms(torch, fn, reps, stream):
    fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def run_k_rhs(args, dev):
    """128^3 constant 7-point Laplacian, 32 right-hand sides N(0,1) in one PCG
    (n x 32 row-major) against 32 single-vector solves; FP32 G."""
    import torch

    import rchol_gb300 as R
    from rchol_gb300 import _lib, generators

    L = _lib.lib()
    A = generators.laplace_3d(128)
    n, k = A.shape[0], 32
    tree = R.Tree.build(A.indptr, A.indices, 256)
    Ad = R.Matrix.create(A.indptr, A.indices, A.data, tree)
    F = R.Factor.compute(Ad, tree, seed=args.seed, precision=R.PREC_FP32)
    B = torch.tensor(np.random.default_rng(args.seed + 7).standard_normal((n, k)), device=dev)
    X = torch.zeros_like(B)
    b1 = B[:, 0].contiguous()
    x1 = torch.zeros_like(b1)
    rr = np.zeros(k)
    it = np.zeros(k, dtype=np.int32)
    stream = torch.cuda.current_stream(dev)
    st = stream.cuda_stream

    def solve(b, x, kk):
        _lib.check(L.rchol_gpu_pcg_d(Ad.ptr, F.ptr, b.data_ptr(), x.data_ptr(), kk, args.tol, args.maxit,
                                     _lib.pd(rr), it.ctypes.data_as(_lib._ip), st))

    t1 = _event_ms(torch, lambda: solve(b1, x1, 1), 3, stream)
    it1 = int(it[0])
    tk = _event_ms(torch, lambda: solve(B, X, k), 2, stream)
    Xh = X.cpu().numpy()
    Bh = B.cpu().numpy()
    perm, _ = tree.arrays()
    Ap = A[perm][:, perm].tocsr()
    worst = float(max(np.linalg.norm(Ap @ Xh[:, j] - Bh[:, j]) / np.linalg.norm(Bh[:, j]) for j in range(k)))
    return {"workload": "PCG to 1e-8, 7-point constant Laplacian 128^3 (n=2,097,152), 32 right-hand sides, FP32 G",
            "ms_single_rhs": round(t1, 2), "iters_single": it1, "ms_32_rhs": round(tk, 2),
            "iters_32": [int(it.min()), int(it.max())], "relres_host_fp64_worst": worst,
            "per_rhs_throughput_vs_single": round(t1 * k / tk, 2)}


def run_batched(args, dev):
    """512 independent 2D 5-point Dirichlet grids, side ~ U{32..256}, edge
    weights exp(0.5 N(0,1)), one N(0,1) right-hand side each, PCG to 1e-8 with
    a block-diagonal FP32 G: all systems in the same launches, against the
    same systems solved one at a time (a sample of 16, extrapolated)."""
    import torch

    import rchol_gb300 as R
    from rchol_gb300 import generators

    rng = np.random.default_rng(args.seed + 11)
    sides = rng.integers(32, 257, 512)
    mats = [generators.grid_2d_weighted(int(sd), int(sd), "lognormal", sigma=0.5, rng=rng) for sd in sides]
    bs = [rng.standard_normal(A.shape[0]) for A in mats]
    t0 = time.time()
    Bt = R.Batch(mats, threads=4, seed=args.seed, precision=R.PREC_FP32)
    torch.cuda.synchronize(dev)
    setup = time.time() - t0
    Bt.solve(bs, args.tol, args.maxit)
    times = []
    for _ in range(3):
        t0 = time.perf_counter()
        xs, relres, itr = Bt.solve(bs, args.tol, args.maxit)
        times.append(time.perf_counter() - t0)
    tb = min(times) * 1e3
    worst = float(max(np.linalg.norm(mats[s] @ xs[s] - bs[s]) / np.linalg.norm(bs[s]) for s in range(len(mats))))
    samp = list(range(0, len(mats), len(mats) // 16))
    tot = 0.0
    for s in samp:
        G, perm, part = R.rchol(mats[s], 4, seed=args.seed, precision="fp32")
        Aps = mats[s][perm][:, perm]
        R.pcg(Aps, bs[s][perm], args.tol, args.maxit, G)
        t0 = time.perf_counter()
        R.pcg(Aps, bs[s][perm], args.tol, args.maxit, G)
        tot += time.perf_counter() - t0
    one = tot / len(samp) * 1e3
    return {"workload": "512 2D 5-point Dirichlet grids, side U{32..256} (n=%d), log-normal(0.5) weights, "
                        "PCG to 1e-8, block-diagonal FP32 G, host buffers" % int(Bt.sys_ptr[-1]),
            "ms_all_systems": round(tb, 1), "iters": [int(itr.min()), int(itr.max())],
            "relres_host_fp64_worst": worst, "setup_s": round(setup, 1),
            "ms_per_system_one_at_a_time": round(one, 2),
            "speedup_vs_one_at_a_time": round(one * len(mats) / tb, 1)}


def run_differentiation(args, dev):
    """2D 5-point weighted Laplacian on a 1024^2 grid, edge weights
    log-uniform in [1e-2, 1e2], diagonal shift 1e-4, b and x_target ~ N(0,1);
    loss 0.5 ||x - x_target||^2 with x = A^-1 b.  Times the forward PCG and
    the backward pass (adjoint PCG with the same G, then the edge-gradient
    kernel for all ~2.1M weights) and checks, on the host in FP64, both
    residuals and dL/dw_e = -(lambda_i - lambda_j)(x_i - x_j) from the
    returned x and lambda = dL/db.  (Finite differences and the dense-solve
    gradient are checked on smaller grids by the tests.)"""
    import torch

    from rchol_gb300.autograd import LaplacianOperator, laplacian_solve

    nx, tol, maxit = 1024, 1e-10, 5000
    rng = np.random.default_rng(args.seed + 23)
    idx = np.arange(nx * nx).reshape(nx, nx)
    ei = np.concatenate([idx[:-1, :].ravel(), idx[:, :-1].ravel()])
    ej = np.concatenate([idx[1:, :].ravel(), idx[:, 1:].ravel()])
    w0 = 10.0 ** rng.uniform(-2.0, 2.0, len(ei))
    b0 = rng.standard_normal(nx * nx)
    xt0 = rng.standard_normal(nx * nx)
    t0 = time.time()
    op = LaplacianOperator(nx * nx, ei, ej, shift=1e-4, nt=256)
    setup = time.time() - t0

    def step():
        w = torch.tensor(w0, device=dev, requires_grad=True)
        b = torch.tensor(b0, device=dev, requires_grad=True)
        xt = torch.tensor(xt0, device=dev)
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        torch.cuda.synchronize(dev)
        e0.record()
        x = laplacian_solve(w, b, op, tol=tol, maxit=maxit)
        e1.record()
        it_f = int(op.last_iters[0])
        loss = 0.5 * ((x - xt) ** 2).sum()
        loss.backward()
        e2.record()
        torch.cuda.synchronize(dev)
        return w, b, x, e0.elapsed_time(e1), e1.elapsed_time(e2), it_f, int(op.last_iters[0])

    t0 = time.time()
    step()  # factors A(w) once (ordering and G are then reused)
    torch.cuda.synchronize(dev)
    factor_s = time.time() - t0
    w, b, x, ms_f, ms_b, it_f, it_b = step()
    A = op.matrix(w0)
    xh = x.detach().cpu().numpy()
    lam = b.grad.cpu().numpy()
    gw = w.grad.cpu().numpy()
    rel_x = float(np.linalg.norm(A @ xh - b0) / np.linalg.norm(b0))
    rel_l = float(np.linalg.norm(A @ lam - (xh - xt0)) / np.linalg.norm(xh - xt0))
    g_host = -(lam[ei] - lam[ej]) * (xh[ei] - xh[ej])
    g_err = float(np.abs(gw - g_host).max() / np.abs(g_host).max())
    ref = differentiation_reference(A, b0, xt0, w0, ei, ej, gw, lam, rng)
    return {"workload": "2D 5-point 1024^2 (n=1,048,576, 2,095,104 edges), log-uniform weights [1e-2, 1e2], "
                        "shift 1e-4, loss 0.5||x - x_target||^2, FP64 G, PCG to 1e-10",
            "ms_forward": round(ms_f, 2), "iters_forward": it_f,
            "ms_backward": round(ms_b, 2), "iters_adjoint": it_b,
            "relres_host_fp64_x": rel_x, "relres_host_fp64_adjoint": rel_l,
            "edge_grad_vs_host_formula": g_err, "independent_check": ref,
            "setup_s": round(setup, 1), "first_step_with_factor_s": round(factor_s, 1)}


def differentiation_reference(A, b, xt, w, ei, ej, gw, lam_gpu, rng, samples=200, rel_step=1e-6):
    """An independent reference for the 1024^2 gradient: one sparse LU of
    A(w) (scipy SuperLU) gives x and lambda = A^-1 (x - x_target) by direct
    solves.  (1) dL/db = lambda and dL/dw_e = -(lambda_i - lambda_j)(x_i - x_j)
    from the LU solves, on all of b and on `samples` random edges, against
    the GPU's adjoint-PCG gradients.  (2) FP64 central finite differences of
    the loss on the same edges, step h = rel_step * w_e: a change of one edge
    weight is the rank-one update A + h d d^T (d = u_i - u_j), so each
    perturbed solve is exact through Sherman-Morrison with z = A^-1 d (one LU
    solve per edge), and L(w + h) - L(w - h) is formed from the two updates
    without cancellation against L itself."""
    import scipy.sparse.linalg as spla

    t0 = time.time()
    lu = spla.splu(A.tocsc(), permc_spec="MMD_AT_PLUS_A")
    x = lu.solve(b)
    r = x - xt
    lam = lu.solve(r)
    pick = rng.choice(len(ei), samples, replace=False)
    gi, gj = ei[pick], ej[pick]
    g_lu = -(lam[gi] - lam[gj]) * (x[gi] - x[gj])
    fd = np.zeros(samples)
    n = A.shape[0]
    for k in range(samples):
        d = np.zeros(n)
        d[gi[k]], d[gj[k]] = 1.0, -1.0
        z = lu.solve(d)
        dx, dz = x[gi[k]] - x[gj[k]], z[gi[k]] - z[gj[k]]
        h = rel_step * w[pick[k]]
        zr, zz = float(z @ r), float(z @ z)
        dL = []
        for sgn in (1.0, -1.0):
            c = sgn * h * dx / (1.0 + sgn * h * dz)  # x(w +- h) = x - c z
            dL.append(-c * zr + 0.5 * c * c * zz)      # L(w +- h) - L(w)
        fd[k] = (dL[0] - dL[1]) / (2 * h)
    scale = np.abs(g_lu).max()
    return {"edges": samples, "fd_rel_step": rel_step, "lu_s": round(time.time() - t0, 1),
            "relres_lu_x": float(np.linalg.norm(A @ x - b) / np.linalg.norm(b)),
            "grad_b_vs_lu": float(np.linalg.norm(lam_gpu - lam) / np.linalg.norm(lam)),
            "grad_w_vs_lu": float(np.abs(gw[pick] - g_lu).max() / scale),
            "grad_w_vs_fd": float(np.abs(gw[pick] - fd).max() / scale),
            "lu_vs_fd": float(np.abs(g_lu - fd).max() / scale)}


def run_c5(args, rank, local):
    """The large high-contrast configuration: 7-point Laplacian on an n^3 grid
    whose cell coefficients form a checkerboard of 1 and 1e4 in 8^3-cell
    blocks (Dirichlet boundary), k = 8 right-hand sides N(0,1), FP32 G, block
    PCG to --tol.  Reports each phase's time, the iterations, the FP64
    host-recomputed residual of every right-hand side, the device memory in
    use at its peak (nvidia-smi) against 180 GB, and the host's peak resident
    memory (this process; the largest forked ordering worker)."""
    import resource

    import torch

    import rchol_gb300 as R
    from rchol_gb300 import _lib, generators

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    L = _lib.lib()
    k = 8
    times = {}
    marks = [("start", time.time())]
    with MemSampler(local) as mem:
        time.sleep(1.0)  # samples before any allocation
        t0 = time.time()
        A = generators.checkerboard_3d(args.n, block=8, lo=1.0, hi=1e4)
        n = A.shape[0]
        times["generate"] = time.time() - t0
        marks.append(("generate", time.time()))
        leaves = args.leaves if args.leaves > 0 else max(1, 2048 * (n // (256 ** 3)))  # ~8,200-row subdomains
        t0 = time.time()
        tree = R.Tree.build(A.indptr, A.indices, leaves)
        perm, _ = tree.arrays()
        times["order"] = time.time() - t0
        marks.append(("order", time.time()))
        t0 = time.time()
        Ad = R.Matrix.create(A.indptr, A.indices, A.data, tree)
        torch.cuda.synchronize()
        times["upload"] = time.time() - t0
        marks.append(("upload", time.time()))
        t0 = time.time()
        F = R.Factor.compute(Ad, tree, seed=args.seed, precision=R.PREC_FP32)
        torch.cuda.synchronize()
        times["factor_gpu"] = time.time() - t0
        marks.append(("factor_gpu", time.time()))
        nnzG = F.nnz
        g = torch.Generator(device=dev)
        g.manual_seed(args.seed + 5)
        B = torch.randn((n, k), generator=g, dtype=torch.float64, device=dev)  # rows in the permuted order
        X = torch.zeros_like(B)
        rr = np.zeros(k)
        it = np.zeros(k, dtype=np.int32)
        stream = torch.cuda.current_stream(dev)

        def solve():
            _lib.check(L.rchol_gpu_pcg_d(Ad.ptr, F.ptr, B.data_ptr(), X.data_ptr(), k, args.tol, args.maxit,
                                         _lib.pd(rr), it.ctypes.data_as(_lib._ip), stream.cuda_stream))

        t0 = time.time()
        solve()  # first call: captures the iteration graph
        torch.cuda.synchronize()
        times["first_solve"] = time.time() - t0
        marks.append(("first_solve", time.time()))
        ms = _event_ms(torch, solve, max(1, args.steps), stream)
        marks.append(("timed_solves", time.time()))
        time.sleep(0.5)
    # FP64 host residuals in the caller's order: x(perm) = X, b(perm) = B
    Xh, Bh = X.cpu().numpy(), B.cpu().numpy()
    worst = 0.0
    for j in range(k):
        x = np.empty(n)
        b = np.empty(n)
        x[perm] = Xh[:, j]
        b[perm] = Bh[:, j]
        worst = max(worst, float(np.linalg.norm(A @ x - b) / np.linalg.norm(b)))
    return {
        "config": "c5",
        "workload": f"block PCG to {args.tol:g}, k={k}, 7-point Laplacian {args.n}^3 (n={n}, nnz(A)={A.nnz}), "
                    f"checkerboard of 1 and 1e4 in 8^3-cell blocks, Dirichlet boundary, FP32 G, {leaves} subdomains",
        "ms_per_solve": round(ms, 1), "unit": "ms", "steps": max(1, args.steps),
        "iters": [int(it.min()), int(it.max())], "relres_gpu_max": float(rr.max()),
        "relres_host_fp64_worst": worst, "nnz_G": int(nnzG),
        "setup_s": {kk: round(v, 2) for kk, v in times.items()},
        "peak_device_gb": mem.peak_gb(), "device_budget_gb": 180,
        "peak_device_gb_by_phase": {marks[i][0]: mem.peak_gb(marks[i - 1][1], marks[i][1]) for i in range(1, len(marks))},
        "device_gb_before_start": mem.peak_gb(marks[0][1] - 1.0, marks[0][1] + 0.9),
        "peak_host_rss_gb": round(resource.getrusage(resource.RUSAGE_SELF).ru_maxrss * 1024 / 1e9, 2),
        "peak_host_rss_child_gb": round(resource.getrusage(resource.RUSAGE_CHILDREN).ru_maxrss * 1024 / 1e9, 2),
    }


def cpu_baseline(args, Ap, bp, F64, it64):
    """The oracle restatement of the reference pcg (pinned bit for bit to the
    reference) on the host cores with the GPU's FP64 factor.  Bounded sample:
    one call that stops before the first iteration (the per-call set-up --
    copies of A and G, the initial and final residuals) and one of S
    iterations; a full solve is then the set-up plus the per-iteration time
    times the FP64 solve's iteration count (no set-up repaid per iteration)."""
    import oracle

    O = oracle.Oracle()
    threads = os.cpu_count() or 1
    rp, ci, v = F64.export()
    G = (rp.astype(np.uint64), ci.astype(np.uint64), v)
    A3 = (Ap.indptr.astype(np.uint64), Ap.indices.astype(np.uint64), Ap.data)
    S = args.cpu_sample_iters
    t0 = time.perf_counter()
    O.pcg(A3, bp, 1e-300, 0, G, threads=threads)
    t_setup = time.perf_counter() - t0
    t0 = time.perf_counter()
    _, _, it = O.pcg(A3, bp, 1e-300, S, G, threads=threads)
    t_s = time.perf_counter() - t0
    per_iter = max(t_s - t_setup, 0.0) / max(it, 1)
    value = t_setup + per_iter * it64
    return {"value": round(value * 1e3, 1), "unit": "ms", "cores": threads, "kind": "port",
            "sample": f"the oracle restatement of c++/util/pcg.cpp (serial triangular solves as MKL's trsv "
                      f"without an analysis hint, SpMV/dots on {threads} threads) on the full {args.n}^3 system "
                      f"with the GPU's FP64 G: set-up {t_setup:.2f} s (a 0-iteration call) + "
                      f"{per_iter:.2f} s/iteration (a {S}-iteration call minus the set-up) x the {it64} "
                      f"iterations of the FP64 solve",
            "setup_s": round(t_setup, 2), "s_per_iteration": round(per_iter, 3)}


def reference_factor_stats(args, A, perm, part, Ad, tree, bp, nnz_gpu, it_gpu):
    """nnz(G) and PCG iterations of the reference's factor (the oracle's
    MODE_REF: the reference's mt19937 streams, pinned bit for bit) with the
    GPU arm's ordering and subdomain count, against the GPU factor's.  The
    reference G's iterations come from the GPU PCG in FP64, which the tests
    pin to the reference pcg with identical iteration counts."""
    import oracle

    import rchol_gb300 as R

    O = oracle.Oracle()
    t0 = time.time()
    A3 = (A.indptr.astype(np.uint64), A.indices.astype(np.uint64), A.data)
    Ap = O.reorder(A3, perm.astype(np.uint64))
    G, _, _ = O.factor(O.extend(Ap), part.astype(np.uint64), oracle.MODE_REF, args.seed)
    t_factor = time.time() - t0
    del Ap
    F = R.Factor.from_host(G[0], G[1], G[2], tree)
    nnz_ref = len(G[1])
    del G
    n = len(bp)
    x, relres, itr = R._pcg_host(Ad, F, bp.reshape(n, 1), args.tol, args.maxit)
    it_ref = int(itr[0])
    return {"subdomains": args.leaves, "nnz_gpu": int(nnz_gpu), "nnz_ref": int(nnz_ref),
            "nnz_ratio": round(nnz_gpu / nnz_ref, 4), "iters_gpu_fp64": int(it_gpu), "iters_ref": it_ref,
            "iters_ratio": round(it_gpu / it_ref, 4), "relres_ref_gpu_pcg": float(relres[0]),
            "ref_factor_host_s": round(t_factor, 1)}


# --------------------------------------------------------------------------------------
# reference arm: the reference's CPU implementation (oracle port, pinned bit for bit)
# --------------------------------------------------------------------------------------

def run_reference(args, rank, world):
    """The reference algorithm on the host cores (oracle port pinned bit for
    bit to the reference): its ordering with the GPU arm's subdomain count,
    its factor (mt19937 streams, subtrees on threads as its std::async tree
    does), then whole PCG solves to the tolerance.  Each step is one complete
    solve; the first untimed solve also gives the iteration count.  A whole
    solve takes tens of seconds, so at most two are timed (steps_requested
    records the request)."""
    if rank != 0:
        return None
    import oracle

    O = oracle.Oracle()
    threads = os.cpu_count() or 1
    A, b, _ = build_problem(args)
    if args.leaves <= 0:  # the gb300 arm's count: tuned for this shape, else 2048 (no GPU library needed)
        import json

        try:
            with open(os.path.join(ROOT, "rchol_gb300", "tuning_cache.json")) as f:
                ent = json.load(f).get(f"n={A.shape[0]},nnz={A.nnz},prec=fp32")
        except (OSError, ValueError):
            ent = None
        args.leaves = int(ent["subdomains"]) if ent else 2048
    A3 = (A.indptr.astype(np.uint64), A.indices.astype(np.uint64), A.data)
    t0 = time.time()
    perm, ridx = O.order(A3, args.leaves)
    t_order = time.time() - t0
    Ap = O.reorder(A3, perm)
    t0 = time.time()
    G, d, _ = O.factor(O.extend(Ap), ridx, oracle.MODE_REF, args.seed)
    t_factor = time.time() - t0
    bp = np.ascontiguousarray(b[perm.astype(np.int64)])
    t0 = time.perf_counter()
    _, relres, iters = O.pcg(Ap, bp, args.tol, args.maxit, G, threads=threads)  # untimed warm-up
    t_first = time.perf_counter() - t0
    steps = max(1, min(args.steps, 2))
    t0 = time.perf_counter()
    for _ in range(steps):
        x, relres, iters = O.pcg(Ap, bp, args.tol, args.maxit, G, threads=threads)
    value = (time.perf_counter() - t0) / steps * 1e3
    import scipy.sparse as sp

    Apm = sp.csr_matrix((Ap[2], Ap[1].astype(np.int64), Ap[0].astype(np.int64)), shape=A.shape)
    ver = float(np.linalg.norm(Apm @ x - bp) / np.linalg.norm(bp))
    return {
        "metric": METRIC, "impl": "reference", "value": round(value, 1), "unit": "ms", "n_gpus": world,
        "steps": steps, "steps_requested": args.steps, "warmup": 1, "ms_per_step": round(value, 1),
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
        "data": "synthetic (same seeds as the gb300 arm)",
        "config": {"workload": f"PCG to {args.tol:g}, 7-point log-normal Laplacian {args.n}^3, reference rchol G "
                               f"(nnz={len(G[1])}, {args.leaves} subdomains, the gb300 arm's count)",
                   "grid": args.n, "leaves": args.leaves, "tol": args.tol, "same_config": True},
        "iters": int(iters), "relres": relres, "relres_host_fp64": ver, "nnz_G": int(len(G[1])),
        "first_solve_s": round(t_first, 1), "order_s": round(t_order, 1), "factor_s": round(t_factor, 1),
        "cpu_baseline": {"value": round(value, 1), "unit": "ms", "cores": threads, "kind": "port",
                         "sample": f"{steps} whole PCG solve(s) to {args.tol:g} of the full system (oracle "
                                   f"restatement of c++/util/pcg.cpp: serial triangular solves as MKL's trsv "
                                   f"without an analysis hint, SpMV/dots on {threads} threads)"},
        "e2e": {"value": round(value, 1), "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    args = parse()
    rank, local, world, pg = dist_init(args)
    if args.impl == "reference":
        line = run_reference(args, rank, world)
    elif args.config == "c5":
        line = run_c5(args, rank, local)
    else:
        line = run_gb300(args, rank, local, world, pg)
    if rank == 0 and line is not None:
        print(json.dumps(line), flush=True)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
