"""Factors made elsewhere (the reference's rchol -> pcg call sequence,
c++/ex_laplace_parallel.cpp:33-46, c++/util/pcg.hpp:15-16).

* The C++ drop-in header runs the reference example's GPU calls: rchol with
  a thread count, reorder, pcg with the G it returned (the resident factor)
  and with a copy of that G (not the resident object: loaded from host
  memory, its tree read off the pattern), both converging with the same
  iteration count.
* The reference's own G (the oracle's MODE_REF) loaded without its tree:
  the tree read off G's pattern keeps the parallelism of the ordering's tree
  (sequential block steps within 1.5x), and PCG matches the reference pcg to
  1e-12 with the same iteration count; the solve time against the same G
  loaded with its tree is printed and bounded.
"""

import os
import subprocess
import time

import numpy as np
import pytest

import oracle
from rchol_gb300 import generators
from conftest import ROOT, csr_u64

pytestmark = pytest.mark.gpu


def test_cpp_example_gpu_branch(cuda, R):
    scratch = os.path.join(ROOT, "tests", ".scratch")
    os.makedirs(scratch, exist_ok=True)
    src = os.path.join(scratch, "cpp_example_gpu.cpp")
    with open(src, "w") as f:
        f.write('#include "rchol_gb300.hpp"\n'
                "#include <chrono>\n#include <cstdio>\n#include <vector>\n"
                "int main() {\n"
                "  SparseCSR A = laplace_3d(32);\n"
                "  SparseCSR G;\n"
                "  std::vector<size_t> P;\n"
                "  rchol(A, G, P, 16);\n"
                "  SparseCSR Aperm;\n"
                "  reorder(A, P, Aperm);\n"
                "  std::vector<double> b(A.size()), bp, x, x2;\n"
                "  for (size_t i = 0; i < b.size(); ++i) b[i] = (double)((i * 7919) % 1000) / 500.0 - 1.0;\n"
                "  reorder(b, P, bp);\n"
                "  double r1 = 0, r2 = 0;\n"
                "  int i1 = 0, i2 = 0;\n"
                "  pcg(Aperm, bp, 1e-10, 200, G, x, r1, i1);\n"
                "  std::vector<size_t> rp(G.rowPtr, G.rowPtr + G.N + 1), ci(G.colIdx, G.colIdx + G.nnz());\n"
                "  std::vector<double> v(G.val, G.val + G.nnz());\n"
                "  SparseCSR Gc;\n"
                "  Gc.init(rp, ci, v, true);\n"
                "  pcg(Aperm, bp, 1e-10, 200, Gc, x2, r2, i2);\n"
                "  double d = 0, nx = 0;\n"
                "  for (size_t i = 0; i < x.size(); ++i) { d += (x[i] - x2[i]) * (x[i] - x2[i]); nx += x[i] * x[i]; }\n"
                "  std::printf(\"%d %d %.3e %.3e %.3e\\n\", i1, i2, r1, r2, d / nx);\n"
                "  return (r1 < 1e-10 && r2 < 1e-10 && i1 == i2) ? 0 : 2;\n"
                "}\n")
    exe = os.path.join(scratch, "cpp_example_gpu")
    lib_dir = os.path.join(ROOT, "rchol_gb300")
    subprocess.run(["g++", "-std=c++17", "-O1", src, "-I", os.path.join(ROOT, "include"), "-L", lib_dir,
                    "-lrchol_gb300", f"-Wl,-rpath,{lib_dir}", "-o", exe], check=True)
    res = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stdout + res.stderr
    i1, i2, r1, r2, dx = res.stdout.split()
    assert float(dx) < 1e-20  # the same G, loaded twice: the same iterates to rounding


def test_reference_factor_without_its_tree(cuda, O, R):
    A = generators.laplace_3d(64)
    Au = csr_u64(A)
    tree = R.Tree.build(A.indptr, A.indices, 256)
    perm, part = tree.arrays()
    Ap = O.reorder(Au, perm.astype(np.uint64))
    G, d, singular = O.factor(O.extend(Ap), part.astype(np.uint64), oracle.MODE_REF, 5)  # the reference's G
    F_tree = R.Factor.from_host(G[0], G[1], G[2], tree)
    F_own = R.Factor.from_host(G[0], G[1], G[2])  # no tree: read off the pattern
    for t in (False, True):
        st_tree, st_own = F_tree.plan_info(t)[2], F_own.plan_info(t)[2]
        assert st_own <= 1.5 * st_tree + 8, (t, st_own, st_tree)
    n = A.shape[0]
    b = np.random.default_rng(3).uniform(-1, 1, n)
    bp = np.ascontiguousarray(b[perm])
    Ad = R.Matrix.create(Ap[0].astype(np.int64), Ap[1].astype(np.int64), Ap[2])  # A(p,p), the caller's system
    x, relres, itr = R._pcg_host(Ad, F_own, bp.reshape(n, 1), 1e-10, 200)
    xo, rro, ito = O.pcg(Ap, bp, 1e-10, 200, G)
    assert int(itr[0]) == ito
    assert np.linalg.norm(x[:, 0] - xo) / np.linalg.norm(xo) < 1e-12

    def timed(F):
        R._pcg_host(Ad, F, bp.reshape(n, 1), 1e-10, 200)
        t0 = time.perf_counter()
        for _ in range(3):
            R._pcg_host(Ad, F, bp.reshape(n, 1), 1e-10, 200)
        return (time.perf_counter() - t0) / 3 * 1e3

    ms_tree, ms_own = timed(F_tree), timed(F_own)
    print(f"\n64^3 reference G, PCG to 1e-10 ({ito} iterations): with its tree {ms_tree:.2f} ms, "
          f"tree read off G {ms_own:.2f} ms; plan steps fwd {F_tree.plan_info()[2]} / {F_own.plan_info()[2]}")
    assert ms_own <= 1.5 * ms_tree + 2.0


def test_tuner_keeps_results_and_is_not_slower(cuda, R):
    """rchol_gpu_factor_tune: the chosen launch knobs give bit-identical
    preconditioner results (they change scheduling only) and a time no worse
    than the starting choice."""
    import torch

    from rchol_gb300 import _lib

    A = generators.laplace_3d_weighted(48, sigma=1.0, seed=2)
    tree = R.Tree.build(A.indptr, A.indices, 64)
    Ad = R.Matrix.create(A.indptr, A.indices, A.data, tree)
    for prec in (R.PREC_FP32, R.PREC_FP64):
        F = R.Factor.compute(Ad, tree, seed=1, precision=prec)
        r = torch.tensor(np.random.default_rng(9).standard_normal(A.shape[0]), device=cuda)
        z0, z1 = torch.empty_like(r), torch.empty_like(r)
        st = torch.cuda.current_stream().cuda_stream
        _lib.check(_lib.lib().rchol_gpu_precond_d(F.ptr, r.data_ptr(), z0.data_ptr(), 1, st))
        info = F.tune()
        _lib.check(_lib.lib().rchol_gpu_precond_d(F.ptr, r.data_ptr(), z1.data_ptr(), 1, st))
        torch.cuda.synchronize()
        assert torch.equal(z0, z1)
        assert info["ms_after"] <= info["ms_before"], info
