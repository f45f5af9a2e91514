"""Golden vectors for the Python front end's ordering.

Compiles the reference's own Cython `find_separator` (python/rchol_lap/
find_separator.pyx with metis_separator.cpp, unmodified) against the METIS
archive of the CUDA toolkit into oracle/_ref/pyref/, runs it the way
python/rchol/rchol.py:31-33 does (A minus its diagonal, depth 1 to
log2(nt) + 1) and stores perm and part (with the ground vertex added to the
last part, rchol.py:33-34) in tests/golden/python_order.npz.

Run in the development container (needs the reference sources and cython):
    python tests/golden/make_python_order.py
"""

import glob
import importlib.util
import math
import os
import shutil
import subprocess
import sys
import sysconfig

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF = os.path.join(os.environ.get("RCHOL_REFERENCE_DIR", "/root/reference"), "python", "rchol_lap")
OUT = os.path.join(ROOT, "oracle", "_ref", "pyref")
CASES = [(8, 2), (10, 4), (12, 8), (16, 16), (20, 32)]


def build():
    os.makedirs(OUT, exist_ok=True)
    for f in ("find_separator.pyx", "metis_separator.cpp"):
        shutil.copy(os.path.join(REF, f), OUT)
    subprocess.run(["cython", "--cplus", "-3", "find_separator.pyx", "-o", "find_separator.cpp"], cwd=OUT, check=True)
    metis = sorted(glob.glob("/usr/local/cuda/targets/*/lib/libmetis_static.a"))[0]
    import numpy

    so = "find_separator" + sysconfig.get_config_var("EXT_SUFFIX")
    subprocess.run(["g++", "-O2", "-shared", "-fPIC", "-std=c++17", "-I", os.path.join(ROOT, "oracle", "shim"), "-I",
                    OUT, "-I", sysconfig.get_paths()["include"], "-I", numpy.get_include(), "find_separator.cpp", metis,
                    "-o", so], cwd=OUT, check=True)
    spec = importlib.util.spec_from_file_location("find_separator", os.path.join(OUT, so))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def main():
    sys.path.insert(0, ROOT)
    from rchol_gb300.generators import laplace_3d

    fs = build()
    out = {}
    for n, nt in CASES:
        A = laplace_3d(n)
        D = sp.diags(A.diagonal(), format="csr")
        perm, val, _ = fs.find_separator(sp.csr_matrix(A - D), 1, math.log2(nt) + 1)
        part = np.append(0, np.cumsum(val)).astype(np.int64)
        part[-1] += 1
        out[f"perm_{n}_{nt}"] = np.asarray(perm, dtype=np.int64)
        out[f"part_{n}_{nt}"] = part
    np.savez_compressed(os.path.join(HERE, "python_order.npz"), **out)
    print("wrote", os.path.join(HERE, "python_order.npz"), sorted(out))


if __name__ == "__main__":
    main()
