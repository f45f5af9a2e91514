"""Autotuning of the single-system path.

Two levels:

* launch choices of the triangular solves on a given factor
  (``Factor.tune()``, rchol_gpu_factor_tune): L2 prefetch distance and ring
  depth of the pipeline format, warps per thread block and prefetch of the
  warp format -- scheduling only, the results are bit-identical;
* the number of nested-dissection subdomains (the reference's ``threads``,
  c++/rchol/rchol_parallel.cpp:39-43), which changes the ordering, G and the
  iteration count: ``tune_subdomains`` orders, factors and solves the system
  once per candidate and keeps the fastest whole PCG solve.

Choices are cached per matrix shape (n, nnz, precision) in
``tuning_cache.json`` beside this file, which ``subdomains_for`` reads.
"""

from __future__ import annotations

import json
import os
import time

import numpy as np

from . import _lib
from ._lib import PREC_FP32, Factor, Matrix, Tree

CACHE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tuning_cache.json")


def _key(n, nnz, precision):
    return f"n={int(n)},nnz={int(nnz)},prec={'fp32' if precision == PREC_FP32 else 'fp64'}"


def load_cache(path=CACHE):
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def subdomains_for(n, nnz, precision=PREC_FP32, default=2048, path=CACHE):
    """The cached subdomain count for this shape, else `default`."""
    ent = load_cache(path).get(_key(n, nnz, precision))
    return int(ent["subdomains"]) if ent else int(default)


def tune_subdomains(A, b, candidates=(1024, 2048, 4096), precision=PREC_FP32, tol=1e-8, maxit=200, seed=0,
                    path=CACHE, write=True):
    """Order, factor and solve A x = b (permuted) once per candidate subdomain
    count, with the launch choices tuned on each factor; keep the fastest
    whole PCG solve (CUDA events, device-resident vectors) and cache it."""
    import torch

    L = _lib.lib()
    n = A.shape[0]
    results = {}
    for t in candidates:
        tree = Tree.build(A.indptr, A.indices, int(t))
        perm, _ = tree.arrays()
        Ad = Matrix.create(A.indptr, A.indices, A.data, tree)
        F = Factor.compute(Ad, tree, seed=seed, precision=precision)
        knobs = F.tune()
        db = torch.tensor(np.ascontiguousarray(b[perm]), dtype=torch.float64, device="cuda")
        dx = torch.zeros_like(db)
        rr = np.zeros(1)
        it = np.zeros(1, dtype=np.int32)
        stream = torch.cuda.current_stream()

        def solve():
            _lib.check(L.rchol_gpu_pcg_d(Ad.ptr, F.ptr, db.data_ptr(), dx.data_ptr(), 1, tol, maxit, _lib.pd(rr),
                                         it.ctypes.data_as(_lib._ip), stream.cuda_stream))

        solve()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(3):
            solve()
        e1.record(stream)
        torch.cuda.synchronize()
        results[int(t)] = {"ms": e0.elapsed_time(e1) / 3, "iters": int(it[0]), "nnz_G": int(F.nnz),
                           "knobs": knobs}
        del F, Ad, tree
    best = min(results, key=lambda t: results[t]["ms"])
    entry = {"subdomains": best, "results": {str(k): v for k, v in results.items()}, "tol": tol,
             "tuned_at": time.strftime("%Y-%m-%d")}
    if write:
        cache = load_cache(path)
        cache[_key(n, A.nnz, precision)] = entry
        with open(path, "w") as f:
            json.dump(cache, f, indent=1, sort_keys=True)
    return entry
