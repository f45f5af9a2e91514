"""GPU triangular solves, SpMV and PCG (through the C ABI) against the
reference's own factor G and the reference PCG (via the pinned oracle and the
golden fixtures): 1e-12 relative in FP64 and identical iteration counts."""

import os

import numpy as np
import pytest

import oracle
from rchol_gb300 import _lib, generators
from conftest import GOLDEN, csr_u64, load_golden

pytestmark = pytest.mark.gpu

TOL = 1e-12  # relative, FP64 path


def _dev(torch, a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def _stream(torch):
    return torch.cuda.current_stream().cuda_stream


def _spread(O, Ap, b, tol, maxit, G, xo):
    """How far the reference PCG itself moves (relative, after `maxit`
    iterations) when nothing but the FP64 rounding order changes: its dot
    products on 8 threads, and additionally its triangular solves in the other
    valid evaluation order.  CG on an ill-conditioned system amplifies such
    rounding differences; this is the reproducibility floor of the case."""
    s = 0.0
    for threads in (8, -8):
        x, _, it = O.pcg(Ap, b, tol, maxit, G, threads=threads)
        s = max(s, np.linalg.norm(x - xo) / np.linalg.norm(xo))
    return s


def _relres_tol(Ap, x, xo, b):
    """Largest |relres - relres_ref| that x and the reference iterate xo allow:
    | ||Ax-b|| - ||Axo-b|| | <= ||A(x-xo)||, plus the rounding of forming each
    residual (a few ulps of |A||x| + |b|), all over ||b||."""
    import scipy.sparse as sp

    n = len(Ap[0]) - 1
    A = sp.csr_matrix((Ap[2], np.asarray(Ap[1], np.int64), np.asarray(Ap[0], np.int64)), shape=(n, n))
    nb = np.linalg.norm(b)
    rounding = 16 * np.finfo(float).eps * np.linalg.norm(abs(A) @ np.abs(x) + np.abs(b))
    return (np.linalg.norm(A @ (x - xo)) + 2 * rounding) / nb


@pytest.mark.parametrize("path", GOLDEN, ids=lambda p: os.path.basename(p)[:-4])
def test_golden_pcg(cuda, O, R, path):
    """Reference G + reference pcg outputs, straight from the golden fixtures.
    The converged iterate must agree within max(1e-12, 4x the spread the
    reference algorithm itself shows when only its rounding order changes)
    -- CG's FP64 reproducibility floor on ill-conditioned cases."""
    g = load_golden(path)
    n = len(g["Ap_rp"]) - 1
    threads = int(g["threads"])
    tree = R.Tree.from_partition(g["perm"].astype(np.int64), g["ridx"].astype(np.int64)) if threads else None
    Ad = R.Matrix.create(g["Ap_rp"], g["Ap_ci"], g["Ap_v"])
    F = R.Factor.from_host(g["G_rp"], g["G_ci"], g["G_v"], tree)
    x, relres, itr = R._pcg_host(Ad, F, g["b"].reshape(n, 1), float(g["tol"]), 200)
    assert int(itr[0]) == int(g["itr"])
    Ap = (g["Ap_rp"], g["Ap_ci"], g["Ap_v"])
    G = (g["G_rp"], g["G_ci"], g["G_v"])
    spread = _spread(O, Ap, g["b"], float(g["tol"]), 200, G, g["x"])
    assert np.linalg.norm(x[:, 0] - g["x"]) / np.linalg.norm(g["x"]) < max(TOL, 4 * spread)
    # ||Ax-b|| of a converged solve is a difference of near-equal terms: it
    # may differ by what the difference of the iterates allows
    assert abs(relres[0] - float(g["relres"])) <= _relres_tol(Ap, x[:, 0], g["x"], g["b"])


CASES = [
    ("lap16_t8", lambda: generators.laplace_3d(16), 8, 1e-10),
    ("lap24_t64", lambda: generators.laplace_3d(24), 64, 1e-10),
    ("weighted14_t16", lambda: generators.laplace_3d_weighted(14, sigma=1.0, seed=1), 16, 1e-8),
    ("grid2d_t16", lambda: generators.grid_2d_weighted(64, 48, "loguniform", shift=1e-4, dirichlet=False, seed=4), 16, 1e-8),
]


@pytest.fixture(scope="module", params=CASES, ids=[c[0] for c in CASES])
def case(request, cuda, O, R):
    name, make, threads, tol = request.param
    A = make()
    Au = csr_u64(A)
    G, perm, ridx, d = O.rchol(Au, threads, seed=31, mode=oracle.MODE_REF)  # == the reference's G
    Ap = O.reorder(Au, perm)
    tree = R.Tree.from_partition(perm.astype(np.int64), ridx.astype(np.int64))
    Ad = R.Matrix.create(A.indptr, A.indices, A.data, tree)
    F = R.Factor.from_host(G[0], G[1], G[2], tree)
    return dict(A=A, Ap=Ap, G=G, perm=perm, tree=tree, Ad=Ad, F=F, tol=tol, n=A.shape[0])


def test_trsv_forward_backward(case, O):
    import torch

    n = case["n"]
    r = np.random.default_rng(2).standard_normal(n)
    L = _lib.lib()
    dr, dy, dz = _dev(torch, r), torch.empty(n, dtype=torch.float64, device="cuda"), torch.empty(
        n, dtype=torch.float64, device="cuda")
    _lib.check(L.rchol_gpu_trsv_d(case["F"].ptr, 0, dr.data_ptr(), dy.data_ptr(), 1, _stream(torch)))
    _lib.check(L.rchol_gpu_trsv_d(case["F"].ptr, 1, dy.data_ptr(), dz.data_ptr(), 1, _stream(torch)))
    y_o = O.trsv_lower(case["G"], r)
    z_o = O.trsv_upper(case["G"], y_o)
    y, z = dy.cpu().numpy(), dz.cpu().numpy()
    assert np.linalg.norm(y - y_o) / np.linalg.norm(y_o) < TOL
    assert np.linalg.norm(z - z_o) / np.linalg.norm(z_o) < TOL
    _lib.check(L.rchol_gpu_precond_d(case["F"].ptr, dr.data_ptr(), dz.data_ptr(), 1, _stream(torch)))
    zp = dz.cpu().numpy()
    zo = O.precond(case["G"], r)
    assert np.linalg.norm(zp - zo) / np.linalg.norm(zo) < TOL


@pytest.mark.parametrize("k", [2, 32, 40])
def test_trsv_many_rhs(case, O, k):
    """k right-hand sides (n x k row-major; more than 32 run in groups of 32)
    against the oracle's single-vector solves, column by column, both
    directions and the preconditioner, FP64 and FP32 factors."""
    import torch

    n = case["n"]
    Rm = np.random.default_rng(7 + k).standard_normal((n, k))
    L = _lib.lib()
    dr = _dev(torch, Rm)
    dy = torch.empty_like(dr)
    dz = torch.empty_like(dr)
    st = _stream(torch)
    _lib.check(L.rchol_gpu_trsv_d(case["F"].ptr, 0, dr.data_ptr(), dy.data_ptr(), k, st))
    _lib.check(L.rchol_gpu_trsv_d(case["F"].ptr, 1, dr.data_ptr(), dz.data_ptr(), k, st))
    Y, Z = dy.cpu().numpy(), dz.cpu().numpy()
    for j in range(k):
        y_o = O.trsv_lower(case["G"], Rm[:, j].copy())
        z_o = O.trsv_upper(case["G"], Rm[:, j].copy())
        assert np.linalg.norm(Y[:, j] - y_o) / np.linalg.norm(y_o) < TOL, j
        assert np.linalg.norm(Z[:, j] - z_o) / np.linalg.norm(z_o) < TOL, j
    _lib.check(L.rchol_gpu_precond_d(case["F"].ptr, dr.data_ptr(), dz.data_ptr(), k, st))
    Z = dz.cpu().numpy()
    for j in range(k):
        zo = O.precond(case["G"], Rm[:, j].copy())
        assert np.linalg.norm(Z[:, j] - zo) / np.linalg.norm(zo) < TOL, j
    # FP32 factor: the k-vector solve equals the single-vector FP32 solve to FP32 rounding
    G = case["G"]
    R = __import__("rchol_gb300")
    F32 = R.Factor.from_host(G[0], G[1], G[2], case["tree"], precision=R.PREC_FP32)
    _lib.check(L.rchol_gpu_precond_d(F32.ptr, dr.data_ptr(), dz.data_ptr(), k, st))
    Z32 = dz.cpu().numpy()
    z1 = torch.empty(n, dtype=torch.float64, device="cuda")
    for j in (0, k - 1):
        r1 = _dev(torch, Rm[:, j].copy())
        _lib.check(L.rchol_gpu_precond_d(F32.ptr, r1.data_ptr(), z1.data_ptr(), 1, st))
        zs = z1.cpu().numpy()
        assert np.linalg.norm(Z32[:, j] - zs) / np.linalg.norm(zs) < 1e-5, j


def test_spmv(case, O):
    import torch

    n = case["n"]
    x = np.random.default_rng(3).standard_normal(n)
    dx, dy = _dev(torch, x), torch.empty(n, dtype=torch.float64, device="cuda")
    _lib.check(_lib.lib().rchol_gpu_spmv_d(case["Ad"].ptr, dx.data_ptr(), dy.data_ptr(), 1, _stream(torch)))
    yo = O.spmv(case["Ap"], x)
    assert np.abs(dy.cpu().numpy() - yo).max() <= 1e-13 * np.abs(yo).max()


def test_pcg_matches_reference_iterates(case, O, R):
    """Iterates after 1, 3, 7 steps and at convergence match the reference
    PCG to 1e-12, or, on the ill-conditioned cases, within 4x the spread the
    reference algorithm itself shows when only its dot-product summation order
    changes (CG's FP64 reproducibility floor)."""
    n = case["n"]
    b = np.random.default_rng(4).uniform(-1, 1, n)
    bp = b[case["perm"].astype(np.int64)]
    for maxit in (1, 3, 7, 200):
        x, relres, itr = R._pcg_host(case["Ad"], case["F"], bp.reshape(n, 1), case["tol"], maxit)
        xo, rro, ito = O.pcg(case["Ap"], bp, case["tol"], maxit, case["G"])
        assert int(itr[0]) == ito
        err = np.linalg.norm(x[:, 0] - xo) / np.linalg.norm(xo)
        spread = _spread(O, case["Ap"], bp, case["tol"], maxit, case["G"], xo)
        assert err < max(TOL, 4 * spread), (maxit, err, spread)
        assert abs(relres[0] - rro) <= _relres_tol(case["Ap"], x[:, 0], xo, bp)


def test_pcg_multi_rhs(case, O, R):
    n, k = case["n"], 5
    B = np.random.default_rng(5).standard_normal((n, k))
    X, relres, itr = R._pcg_host(case["Ad"], case["F"], B, case["tol"], 200)
    for j in range(k):
        xo, rro, ito = O.pcg(case["Ap"], B[:, j].copy(), case["tol"], 200, case["G"])
        spread = _spread(O, case["Ap"], B[:, j].copy(), case["tol"], 200, case["G"], xo)
        assert int(itr[j]) == ito
        assert np.linalg.norm(X[:, j] - xo) / np.linalg.norm(xo) < max(TOL, 4 * spread)


def test_fp32_preconditioner(case, O, R):
    """G stored and applied in FP32: error of z against the FP64 oracle and the
    iteration penalty are bounded (stated per case in the assertion message)."""
    n = case["n"]
    G = case["G"]
    F32 = R.Factor.from_host(G[0], G[1], G[2], case["tree"], precision=R.PREC_FP32)
    b = np.random.default_rng(6).uniform(-1, 1, n)
    bp = b[case["perm"].astype(np.int64)]
    x64, rr64, it64 = R._pcg_host(case["Ad"], case["F"], bp.reshape(n, 1), case["tol"], 200)
    x32, rr32, it32 = R._pcg_host(case["Ad"], F32, bp.reshape(n, 1), case["tol"], 200)
    Ap = case["Ap"]
    import scipy.sparse as sp

    Am = sp.csr_matrix((Ap[2], Ap[1].astype(np.int64), Ap[0].astype(np.int64)), shape=(n, n))
    true_rel = np.linalg.norm(Am @ x32[:, 0] - bp) / np.linalg.norm(bp)  # FP64 host check
    assert true_rel <= case["tol"] * 1.01, true_rel
    assert it32[0] <= 1.1 * it64[0] + 1, f"fp32 {it32[0]} vs fp64 {it64[0]} iterations"
    import torch

    r = np.random.default_rng(8).standard_normal(n)
    dr, dz = _dev(torch, r), torch.empty(n, dtype=torch.float64, device="cuda")
    _lib.check(_lib.lib().rchol_gpu_precond_d(F32.ptr, dr.data_ptr(), dz.data_ptr(), 1, _stream(torch)))
    zo = O.precond(G, r)
    err = np.linalg.norm(dz.cpu().numpy() - zo) / np.linalg.norm(zo)
    assert err < 1e-3, f"fp32 preconditioner relative error {err:.2e}"


def test_factor_levels_report_dependency_depth(case):
    """rchol_gpu_factor_levels: the longest dependency chain of the forward
    (rows of G) and backward (rows of G^T) solves, against a host count."""
    Gt_rp, Gt_ci = case["G"][0].astype(np.int64), case["G"][1].astype(np.int64)
    n = len(Gt_rp) - 1
    fwd, bwd = case["F"].levels()
    lv = np.zeros(n, dtype=np.int64)  # backward: row i of G^T depends on its later columns
    for i in range(n - 1, -1, -1):
        cols = Gt_ci[Gt_rp[i] + 1:Gt_rp[i + 1]]
        lv[i] = lv[cols].max() + 1 if cols.size else 0
    assert bwd == lv.max() + 1
    lf = np.zeros(n, dtype=np.int64)  # forward: column j of G^T feeds rows > j
    for j in range(n):
        rows = Gt_ci[Gt_rp[j] + 1:Gt_rp[j + 1]]
        lf[rows] = np.maximum(lf[rows], lf[j] + 1)
    assert fwd == lf.max() + 1
