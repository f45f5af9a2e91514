"""The triangular-solve streams, checked on the CPU.

tests/stream_emulator.cu compiles the library's own stream builder (host
code of rchol_gb300/csrc/trsv.cu) into a CPU program, builds the forward and
backward streams of oracle factors (device-contract mode, i.e. the GPU's G)
and executes them in the kernels' order: every record may only read unknowns
solved at that point, and the result must equal plain substitution.  Warp,
pipeline and staged (warp format for depths with many nodes, pipeline at
the top) formats, FP64 and FP32 values, single and 32-wide records."""

import os
import shutil
import subprocess

import numpy as np
import pytest

import oracle
from rchol_gb300 import generators
from conftest import ROOT, csr_u64

SCRATCH = os.path.join(ROOT, "tests", ".scratch")
NVCC = shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc" if os.path.exists("/usr/local/cuda/bin/nvcc") else None)

CASES = [
    ("lap24_t16", lambda: generators.laplace_3d(24), 16),
    ("weighted20_t8", lambda: generators.laplace_3d_weighted(20, sigma=1.0, seed=4), 8),
    ("grid2d_t8", lambda: generators.grid_2d_weighted(70, 50, "loguniform", shift=1e-4, dirichlet=False, seed=2), 8),
    ("checker16_t8", lambda: generators.checkerboard_3d(16, block=4), 8),
]


@pytest.fixture(scope="module")
def emulator(built):
    if NVCC is None:
        pytest.skip("nvcc not available")
    os.makedirs(SCRATCH, exist_ok=True)
    exe = os.path.join(SCRATCH, "stream_emulator")
    src = os.path.join(ROOT, "tests", "stream_emulator.cu")
    deps = [src] + [os.path.join(ROOT, "rchol_gb300", "csrc", f)
                    for f in ("trsv.cu", "plan.hpp", "common.hpp", "tree_infer.hpp")]
    if not os.path.exists(exe) or os.path.getmtime(exe) < max(os.path.getmtime(d) for d in deps):
        subprocess.run([NVCC, "-std=c++17", "-O2", "-gencode", "arch=compute_103a,code=sm_103a",
                        "-I", os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "rchol_gb300", "csrc"),
                        "-o", exe, src], check=True, capture_output=True)
    return exe


@pytest.fixture(scope="module", params=CASES, ids=[c[0] for c in CASES])
def factor_dir(request, O):
    name, make, threads = request.param
    A = make()
    G, perm, ridx, d = O.rchol(csr_u64(A), threads, seed=7, mode=oracle.MODE_DEVICE)
    out = os.path.join(SCRATCH, name)
    os.makedirs(out, exist_ok=True)
    n = len(G[0]) - 1
    np.array([n, len(G[1]), len(ridx)], np.int64).tofile(os.path.join(out, "hdr.bin"))
    G[0].astype(np.int64).tofile(os.path.join(out, "rp.bin"))
    G[1].astype(np.int32).tofile(os.path.join(out, "ci.bin"))
    np.asarray(G[2], np.float64).tofile(os.path.join(out, "v.bin"))
    np.asarray(ridx, np.int64).tofile(os.path.join(out, "ridx.bin"))
    return out


@pytest.mark.parametrize("fmt,precision,kwidth", [(0, 0, 1), (0, 1, 1), (1, 0, 1), (1, 1, 1), (2, 0, 1), (2, 1, 1),
                                                   (2, 0, 32), (2, 1, 32)],
                         ids=["warp-fp64", "warp-fp32", "staged-fp64", "staged-fp32", "pipe-fp64", "pipe-fp32",
                              "wide-fp64", "wide-fp32"])
def test_streams_solve_exactly(emulator, factor_dir, fmt, precision, kwidth):
    res = subprocess.run([emulator, factor_dir, str(fmt), str(precision), str(kwidth)], capture_output=True,
                         text=True, timeout=300)
    line = res.stdout.strip().splitlines()[-1] if res.stdout.strip() else res.stderr
    assert res.returncode == 0 and line.startswith("ok"), line
    _, rel_fwd, rel_bwd, team_pieces, steps, warp_pieces = line.split()
    tol = 1e-12 if precision == 0 else 1e-4  # FP32 values and arithmetic
    assert float(rel_fwd) < tol and float(rel_bwd) < tol, line
    if fmt == 2:
        assert int(team_pieces) > 0 and int(warp_pieces) == 0
    if fmt == 0 and kwidth == 1:  # depths whose blocks are too dense for a warp's share fall back to the pipeline
        assert int(warp_pieces) > 0


def test_emulator_catches_a_misordered_tree(emulator, O):
    """Negative control, planted on the CPU: the boundary between two sibling
    subdomains is moved so that rows of one read unknowns of the other in the
    same stage; the emulator must refuse the streams."""
    A = generators.laplace_3d(16)
    G, perm, ridx, d = O.rchol(csr_u64(A), 4, seed=7, mode=oracle.MODE_DEVICE)
    out = os.path.join(SCRATCH, "misordered")
    os.makedirs(out, exist_ok=True)
    n = len(G[0]) - 1
    bad = np.asarray(ridx, np.int64).copy()
    bad[1] -= 10  # the last 10 rows of the first subdomain now belong to its sibling
    np.array([n, len(G[1]), len(bad)], np.int64).tofile(os.path.join(out, "hdr.bin"))
    G[0].astype(np.int64).tofile(os.path.join(out, "rp.bin"))
    G[1].astype(np.int32).tofile(os.path.join(out, "ci.bin"))
    np.asarray(G[2], np.float64).tofile(os.path.join(out, "v.bin"))
    bad.tofile(os.path.join(out, "ridx.bin"))
    res = subprocess.run([emulator, out, "2", "0", "1"], capture_output=True, text=True, timeout=300)
    assert res.returncode == 1 and "not yet solved" in res.stdout, res.stdout


def test_inferred_tree_is_exact_and_parallel(emulator, factor_dir):
    """A factor loaded without its tree: the tree read off G's pattern gives
    streams that read only solved unknowns, solve exactly, and keep most of
    the parallelism of the ordering's own tree (sequential block steps within
    1.5x of it, against one chain of n/32 steps without a tree)."""
    runs = {}
    for mode in ("tree", "infer"):
        res = subprocess.run([emulator, factor_dir, "1", "0", "1"] + (["infer"] if mode == "infer" else []),
                             capture_output=True, text=True, timeout=300)
        line = res.stdout.strip().splitlines()[-1] if res.stdout.strip() else res.stderr
        assert res.returncode == 0 and line.startswith("ok"), line
        runs[mode] = line.split()
    _, rel_fwd, rel_bwd, _, steps, _ = runs["infer"]
    assert float(rel_fwd) < 1e-12 and float(rel_bwd) < 1e-12
    n = int(np.fromfile(os.path.join(factor_dir, "hdr.bin"), np.int64)[0])
    assert int(steps) <= 1.5 * int(runs["tree"][4]) + 8, (steps, runs["tree"][4])
    assert int(steps) < 2 * (n + 31) // 32 / 2
