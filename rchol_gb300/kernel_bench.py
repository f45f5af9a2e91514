"""Kernel-level runs for timing and profiling one operation of the solve path.

    python -m rchol_gb300.kernel_bench --n 256 --leaves 2048 --weighted --op trsv --precision fp32 --reps 1

Builds the 7-point Laplacian of an n^3 grid (constant, or with the bench's
log-normal weights), orders it (``leaves`` subdomains), factors it on the GPU
and then runs ``reps`` calls of one operation through the C ABI: a forward
triangular solve (``trsv``), a backward one (``trsv_t``), the preconditioner
(``precond``) or the SpMV (``spmv``).  Prints the mean time per call measured
with CUDA events on the calling stream and the algorithmic bytes per call.
Used for the ncu captures summarised beside the benchmark.
"""

from __future__ import annotations

import argparse

import numpy as np


def main(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, default=64)
    p.add_argument("--leaves", type=int, default=256)
    p.add_argument("--weighted", action="store_true", help="log-normal(1) weights, shift 1e-3 (the bench's matrix)")
    p.add_argument("--op", default="trsv", choices=["trsv", "trsv_t", "precond", "spmv"])
    p.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    p.add_argument("--rhs", type=int, default=1)
    p.add_argument("--reps", type=int, default=1)
    p.add_argument("--tune", action="store_true", help="tune the solves' launch choices first (Factor.tune)")
    args = p.parse_args(argv)

    import torch

    import rchol_gb300 as R
    from rchol_gb300 import _lib, generators

    A = (generators.laplace_3d_weighted(args.n, 1.0, 1e-3, 0) if args.weighted else generators.laplace_3d(args.n))
    n, k = A.shape[0], args.rhs
    tree = R.Tree.build(A.indptr, A.indices, args.leaves)
    Ad = R.Matrix.create(A.indptr, A.indices, A.data, tree)
    prec = R.PREC_FP32 if args.precision == "fp32" else R.PREC_FP64
    F = R.Factor.compute(Ad, tree, seed=0, precision=prec)
    L = _lib.lib()
    stream = torch.cuda.current_stream()
    s = stream.cuda_stream
    x = torch.randn(n * k, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    ops = {
        "trsv": lambda: L.rchol_gpu_trsv_d(F.ptr, 0, x.data_ptr(), y.data_ptr(), k, s),
        "trsv_t": lambda: L.rchol_gpu_trsv_d(F.ptr, 1, x.data_ptr(), y.data_ptr(), k, s),
        "precond": lambda: L.rchol_gpu_precond_d(F.ptr, x.data_ptr(), y.data_ptr(), k, s),
        "spmv": lambda: L.rchol_gpu_spmv_d(Ad.ptr, x.data_ptr(), y.data_ptr(), k, s),
    }
    op = ops[args.op]
    _lib.check(op())  # first call builds the lazily created parts of the plan
    torch.cuda.synchronize()
    if args.tune:
        print("tuned:", F.tune())
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.reps):
        _lib.check(op())
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.reps
    vs = 4 if prec == R.PREC_FP32 else 8
    nnz = F.nnz if args.op != "spmv" else A.nnz
    per_solve = nnz * ((vs if args.op != "spmv" else 8) + 4) + (n + 1) * 8 + 2 * 8 * n * k
    if args.op == "precond":
        per_solve *= 2
    print(f"{args.op} n={n} nnz={nnz} {args.precision} k={k}: {ms:.4f} ms per call, "
          f"{per_solve / 1e9:.4f} GB algorithmic, {per_solve / ms / 1e6:.1f} GB/s")


if __name__ == "__main__":
    main()
