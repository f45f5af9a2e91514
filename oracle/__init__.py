"""ctypes front end for the CPU checkers under oracle/ (test infrastructure).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this package.  It wraps two shared libraries built by oracle/Makefile:

* ``liboracle.so`` -- the restatement of the reference algorithm
  (oracle/rchol_oracle.cpp), available on every machine;
* ``_ref/librchol_ref.so`` -- the unmodified reference C++ compiled from its
  own sources, available only where those sources exist.

All matrices are CSR triples ``(rowptr uint64, colidx uint64, val float64)``.
"""

from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_u64p = C.POINTER(C.c_uint64)
_dp = C.POINTER(C.c_double)
_i64 = C.c_int64

MODE_REF = 0
MODE_DEVICE = 1

# Where the reference sources live (only the development machine has them).
REFERENCE_DIR = os.environ.get("RCHOL_REFERENCE_DIR", "/root/reference")


def build(with_ref: bool | None = None) -> None:
    """Compile liboracle.so (and the reference library if its sources exist)."""
    targets = ["oracle"]
    if with_ref is None:
        with_ref = os.path.isdir(os.path.join(REFERENCE_DIR, "c++"))
    if with_ref:
        targets.append("ref")
    subprocess.run(["make", "-s", "-j8", *targets, f"RCHOL_REFERENCE_DIR={REFERENCE_DIR}"], cwd=HERE, check=True)


def _p(a, t):
    return a.ctypes.data_as(t)


def _u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


class _Lib:
    prefix = ""

    def __init__(self, path):
        self.lib = C.CDLL(path)
        self.free = getattr(self.lib, self.prefix + "free")

    def take(self, ptr, n, dtype):
        a = np.ctypeslib.as_array(ptr, shape=(max(int(n), 1),))[: int(n)].astype(dtype, copy=True)
        self.free(ptr)
        return a

    def take_csr(self, rp, ci, v, n):
        rpa = self.take(rp, n + 1, np.uint64)
        nnz = int(rpa[-1])
        return rpa, self.take(ci, nnz, np.uint64), self.take(v, nnz, np.float64)

    def err(self):
        f = getattr(self.lib, self.prefix + "last_error")
        f.restype = C.c_char_p
        return f().decode()


class Oracle(_Lib):
    """The restatement (liboracle.so)."""

    prefix = "oracle_"

    def __init__(self, path=None):
        path = path or os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build(with_ref=False)
        super().__init__(path)
        self.lib.oracle_uniform.restype = C.c_double
        self.lib.oracle_uniform.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]

    def laplace_3d(self, n):
        rp, ci, v = _u64p(), _u64p(), _dp()
        self.lib.oracle_laplace_3d(_i64(n), C.byref(rp), C.byref(ci), C.byref(v))
        return self.take_csr(rp, ci, v, n ** 3)

    def extend(self, A):
        rp, ci, v = A
        n = len(rp) - 1
        orp, oci, ov = _u64p(), _u64p(), _dp()
        self.lib.oracle_extend(_i64(n), _p(_u64(rp), _u64p), _p(_u64(ci), _u64p), _p(_f64(v), _dp),
                               C.byref(orp), C.byref(oci), C.byref(ov))
        return self.take_csr(orp, oci, ov, n + 1)

    def reorder(self, A, perm):
        rp, ci, v = A
        n = len(rp) - 1
        orp, oci, ov = _u64p(), _u64p(), _dp()
        self.lib.oracle_reorder(_i64(n), _p(_u64(rp), _u64p), _p(_u64(ci), _u64p), _p(_f64(v), _dp),
                                _p(_u64(perm), _u64p), C.byref(orp), C.byref(oci), C.byref(ov))
        return self.take_csr(orp, oci, ov, n)

    def order(self, A, threads, last_in_root=False, leaf_order="natural"):
        """Nested-dissection ordering; last_in_root: the Python front end's
        variant (python/rchol_lap/find_separator.pyx:27-28); leaf_order:
        "natural", "nd" or "md" inside the leaves."""
        rp, ci = A[0], A[1]
        n = len(rp) - 1
        perm, ridx, nr = _u64p(), _u64p(), _i64()
        rc = self.lib.oracle_order_ex(_i64(n), _p(_u64(rp), _u64p), _p(_u64(ci), _u64p), int(threads),
                                      int(bool(last_in_root)) | {"natural": 0, "nd": 2, "md": 4}[leaf_order],
                                      C.byref(perm), C.byref(ridx), C.byref(nr))
        if rc:
            raise ValueError(self.err())
        return self.take(perm, n, np.uint64), self.take(ridx, nr.value, np.uint64)

    def factor(self, L, ridx, mode, seed):
        """Factor an extended Laplacian; returns (G^T CSR triple, pivots d)."""
        rp, ci, v = L
        nx = len(rp) - 1
        ridx = _u64(ridx)
        grp, gci, gv = _u64p(), _u64p(), _dp()
        d = np.zeros(nx)
        rc = self.lib.oracle_factor(_i64(nx), _p(_u64(rp), _u64p), _p(_u64(ci), _u64p), _p(_f64(v), _dp),
                                    _p(ridx, _u64p), _i64(len(ridx)), int(mode), C.c_uint64(seed),
                                    C.byref(grp), C.byref(gci), C.byref(gv), _p(d, _dp))
        if rc == 1:
            raise ValueError(self.err())
        G = self.take_csr(grp, gci, gv, nx - 1)
        return G, d, rc == 2

    def rchol(self, A, threads=0, seed=0, mode=MODE_REF):
        """Whole reference path: order (threads>0), reorder, extend, factor."""
        n = len(A[0]) - 1
        if threads == 0:
            perm = np.arange(n, dtype=np.uint64)
            ridx = np.array([0, n + 1], dtype=np.uint64)
            Ap = A
        else:
            perm, ridx = self.order(A, threads)
            Ap = self.reorder(A, perm)
        G, d, singular = self.factor(self.extend(Ap), ridx, mode, seed)
        return G, perm, ridx, d

    def _g3(self, G):
        return _p(_u64(G[0]), _u64p), _p(_u64(G[1]), _u64p), _p(_f64(G[2]), _dp)

    def precond(self, G, r):
        n = len(G[0]) - 1
        z = np.zeros(n)
        self.lib.oracle_precond(_i64(n), *self._g3(G), _p(_f64(r), _dp), _p(z, _dp))
        return z

    def trsv_lower(self, G, r):
        n = len(G[0]) - 1
        y = np.zeros(n)
        self.lib.oracle_trsv_lower(_i64(n), *self._g3(G), _p(_f64(r), _dp), _p(y, _dp))
        return y

    def trsv_upper(self, G, r):
        n = len(G[0]) - 1
        y = np.zeros(n)
        self.lib.oracle_trsv_upper(_i64(n), *self._g3(G), _p(_f64(r), _dp), _p(y, _dp))
        return y

    def spmv(self, A, x):
        n = len(A[0]) - 1
        y = np.zeros(n)
        self.lib.oracle_spmv(_i64(n), *self._g3(A), _p(_f64(x), _dp), _p(y, _dp))
        return y

    def pcg(self, A, b, tol, maxit, G, threads=1, history=False):
        n = len(A[0]) - 1
        x = np.zeros(n)
        rr = C.c_double()
        it = C.c_int()
        hist = np.zeros(max(maxit, 1))
        self.lib.oracle_pcg(_i64(n), *self._g3(A), _p(_f64(b), _dp), C.c_double(tol), int(maxit),
                            *self._g3(G), int(threads), _p(x, _dp), C.byref(rr), C.byref(it),
                            _p(hist, _dp) if history else None)
        if history:
            return x, rr.value, it.value, hist[: it.value].copy()
        return x, rr.value, it.value

    def philox(self, ctr, key):
        c = np.asarray(ctr, dtype=np.uint32)
        k = np.asarray(key, dtype=np.uint32)
        o = np.zeros(4, dtype=np.uint32)
        u32p = C.POINTER(C.c_uint32)
        self.lib.oracle_philox(_p(c, u32p), _p(k, u32p), _p(o, u32p))
        return o

    def uniform(self, seed, v, i):
        return self.lib.oracle_uniform(seed, v, i)


class Reference(_Lib):
    """The unmodified reference compiled from its sources (oracle/_ref)."""

    prefix = "ref_"
    PATH = os.path.join(HERE, "_ref", "librchol_ref.so")

    @classmethod
    def available(cls):
        return os.path.exists(cls.PATH)

    def __init__(self):
        super().__init__(self.PATH)

    def laplace_3d(self, n):
        N, rp, ci, v = _i64(), _u64p(), _u64p(), _dp()
        self.lib.ref_laplace_3d(int(n), C.byref(N), C.byref(rp), C.byref(ci), C.byref(v))
        return self.take_csr(rp, ci, v, N.value)

    def extend(self, A):
        rp, ci, v = A
        n = len(rp) - 1
        orp, oci, ov = _u64p(), _u64p(), _dp()
        self.lib.ref_extend(_i64(n), _p(_u64(rp), _u64p), _p(_u64(ci), _u64p), _p(_f64(v), _dp),
                            C.byref(orp), C.byref(oci), C.byref(ov))
        return self.take_csr(orp, oci, ov, n + 1)

    def order(self, A, threads):
        rp, ci, v = A
        n = len(rp) - 1
        perm, ridx, nr = _u64p(), _u64p(), _i64()
        rc = self.lib.ref_order(_i64(n), _p(_u64(rp), _u64p), _p(_u64(ci), _u64p), _p(_f64(v), _dp),
                                int(threads), C.byref(perm), C.byref(ridx), C.byref(nr))
        if rc:
            raise ValueError(self.err())
        return self.take(perm, n, np.uint64), self.take(ridx, nr.value, np.uint64)

    def reorder(self, A, perm):
        rp, ci, v = A
        n = len(rp) - 1
        orp, oci, ov = _u64p(), _u64p(), _dp()
        self.lib.ref_reorder(_i64(n), _p(_u64(rp), _u64p), _p(_u64(ci), _u64p), _p(_f64(v), _dp),
                             _p(_u64(perm), _u64p), C.byref(orp), C.byref(oci), C.byref(ov))
        return self.take_csr(orp, oci, ov, n)

    def rchol(self, A, threads=0, seed=0):
        rp, ci, v = A
        n = len(rp) - 1
        grp, gci, gv, pp = _u64p(), _u64p(), _dp(), _u64p()
        rc = self.lib.ref_rchol(_i64(n), _p(_u64(rp), _u64p), _p(_u64(ci), _u64p), _p(_f64(v), _dp),
                                int(threads), C.c_uint(seed), C.byref(grp), C.byref(gci), C.byref(gv),
                                C.byref(pp))
        if rc:
            raise ValueError(self.err())
        G = self.take_csr(grp, gci, gv, n)
        return G, self.take(pp, n, np.uint64)

    def pcg(self, A, b, tol, maxit, G):
        rp, ci, v = A
        n = len(rp) - 1
        x = np.zeros(n)
        rr, it = C.c_double(), C.c_int()
        self.lib.ref_pcg(_i64(n), _p(_u64(rp), _u64p), _p(_u64(ci), _u64p), _p(_f64(v), _dp),
                         _p(_f64(b), _dp), C.c_double(tol), int(maxit), _p(_u64(G[0]), _u64p),
                         _p(_u64(G[1]), _u64p), _p(_f64(G[2]), _dp), _p(x, _dp), C.byref(rr),
                         C.byref(it))
        return x, rr.value, it.value
