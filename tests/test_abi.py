"""The C-ABI library loads, exports every function include/rchol_gpu.h declares,
and the ctypes table matches the header (no GPU calls)."""

import ctypes
import os
import re

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "rchol_gpu.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rchol_gpu_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    from rchol_gb300 import _lib

    lib = ctypes.CDLL(_lib.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_no_unresolved_internal_symbols(built):
    """Every internal function the library calls is defined in it (lazy
    binding would otherwise only fail at the first call, on a GPU)."""
    import subprocess

    from rchol_gb300 import _lib

    out = subprocess.run(["nm", "-D", "-C", "--undefined-only", _lib.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    bad = [ln for ln in out.splitlines() if "rchol" in ln]
    assert not bad, bad
    ctypes.CDLL(_lib.LIB_PATH, mode=os.RTLD_NOW)


def test_ctypes_table_covers_header(built):
    from rchol_gb300 import _lib

    table = {n for n, _, _ in _lib.SIGNATURES}
    assert table == set(declared_functions())


def test_version_and_error_string(built):
    from rchol_gb300 import _lib

    L = _lib.lib()
    assert b"sm_103a" in L.rchol_gpu_version()
    rc = L.rchol_gpu_tree_build(0, None, None, 2, None)
    assert rc == _lib.ERR_INVALID
    assert L.rchol_gpu_last_error()


def test_cpp_header_compiles(built):
    """include/rchol_gb300.hpp (the reference-shaped C++ API) compiles and
    links with the calls of the reference's parallel example
    (c++/ex_laplace_parallel.cpp: laplace_3d, rchol with a permutation and a
    thread count, reorder, pcg); the host-only part runs here, the GPU calls
    are only linked (they run behind a command-line switch)."""
    import subprocess

    scratch = os.path.join(ROOT, "tests", ".scratch")
    os.makedirs(scratch, exist_ok=True)
    src = os.path.join(scratch, "cpp_header.cpp")
    with open(src, "w") as f:
        f.write('#include "rchol_gb300.hpp"\n'
                "#include <vector>\n"
                "int main(int argc, char **argv) {\n"
                "  SparseCSR A = laplace_3d(4);\n"
                "  if (A.size() != 64) return 1;\n"
                "  if (argc > 1) {  // needs a GPU\n"
                "    SparseCSR G;\n"
                "    std::vector<size_t> P;\n"
                "    rchol(A, G, P, 2);\n"
                "    SparseCSR Aperm;\n"
                "    reorder(A, P, Aperm);\n"
                "    std::vector<double> b(A.size(), 1.0), bp, x;\n"
                "    reorder(b, P, bp);\n"
                "    double relres = 0;\n"
                "    int itr = 0;\n"
                "    pcg(Aperm, bp, 1e-10, 100, G, x, relres, itr);\n"
                "    return relres < 1e-10 ? 0 : 2;\n"
                "  }\n"
                "  return 0;\n"
                "}\n")
    exe = os.path.join(scratch, "cpp_header")
    lib_dir = os.path.join(ROOT, "rchol_gb300")
    subprocess.run(["g++", "-std=c++17", "-O1", src, "-I", os.path.join(ROOT, "include"),
                    "-L", lib_dir, "-lrchol_gb300", f"-Wl,-rpath,{lib_dir}", "-o", exe], check=True)
    # laplace_3d and SparseCSR are host-only: running needs no GPU
    assert subprocess.run([exe]).returncode == 0
