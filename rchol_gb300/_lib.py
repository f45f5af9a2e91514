"""ctypes bindings to librchol_gb300.so (the C ABI of include/rchol_gpu.h).

The library is loaded from this package directory; if it is missing the
import fails loudly -- there is no CPU fallback.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "librchol_gb300.so")

OK, ERR_INVALID, ERR_CUDA, ERR_SINGULAR, ERR_NOMEM, ERR_TIMEOUT, ERR_INTERNAL = range(7)
PREC_FP64, PREC_FP32 = 0, 1

_i64 = C.c_int64
_i64p = C.POINTER(C.c_int64)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_vp = C.c_void_p

# (name, restype, argtypes) for every symbol of include/rchol_gpu.h
SIGNATURES = [
    ("rchol_gpu_last_error", C.c_char_p, []),
    ("rchol_gpu_version", C.c_char_p, []),
    ("rchol_gpu_launch_count", _i64, []),
    ("rchol_gpu_tree_build", C.c_int, [_i64, _i64p, _i64p, C.c_int, C.POINTER(_vp)]),
    ("rchol_gpu_tree_build_ex", C.c_int, [_i64, _i64p, _i64p, C.c_int, C.c_int, C.POINTER(_vp)]),
    ("rchol_gpu_tree_build_batch", C.c_int, [_i64, _i64p, _i64, _i64p, _i64p, C.c_int, C.POINTER(_vp)]),
    ("rchol_gpu_tree_from_partition", C.c_int, [_i64, _i64p, _i64p, _i64, C.POINTER(_vp)]),
    ("rchol_gpu_tree_size", _i64, [_vp]),
    ("rchol_gpu_tree_num_parts", _i64, [_vp]),
    ("rchol_gpu_tree_get", C.c_int, [_vp, _i64p, _i64p]),
    ("rchol_gpu_tree_destroy", None, [_vp]),
    ("rchol_gpu_reorder", C.c_int, [_i64, _i64p, _i64p, _dp, _i64p, _i64p, _i64p, _dp]),
    ("rchol_gpu_matrix_create", C.c_int, [_i64, _i64p, _i64p, _dp, _vp, C.POINTER(_vp)]),
    ("rchol_gpu_matrix_size", _i64, [_vp]),
    ("rchol_gpu_matrix_nnz", _i64, [_vp]),
    ("rchol_gpu_matrix_set_values", C.c_int, [_vp, _dp]),
    ("rchol_gpu_matrix_destroy", None, [_vp]),
    ("rchol_gpu_factor", C.c_int, [_vp, _vp, C.c_uint64, C.c_int, C.POINTER(_vp)]),
    ("rchol_gpu_factor_from_host", C.c_int, [_i64, _i64p, _i64p, _dp, _vp, C.c_int, C.POINTER(_vp)]),
    ("rchol_gpu_factor_nnz", _i64, [_vp]),
    ("rchol_gpu_factor_precision", C.c_int, [_vp]),
    ("rchol_gpu_factor_export", C.c_int, [_vp, _i64p, _i64p, _dp]),
    ("rchol_gpu_factor_pivots", C.c_int, [_vp, _dp]),
    ("rchol_gpu_factor_levels", C.c_int, [_vp, _i64p, _i64p]),
    ("rchol_gpu_factor_setup_times", C.c_int, [_vp, _dp, _dp, _dp]),
    ("rchol_gpu_factor_plan_info", C.c_int, [_vp, C.c_int, _i64p, _i64p, _i64p]),
    ("rchol_gpu_factor_tune", C.c_int, [_vp, _dp, _dp, C.POINTER(C.c_int)]),
    ("rchol_gpu_factor_destroy", None, [_vp]),
    ("rchol_gpu_pcg", C.c_int, [_vp, _vp, _dp, _dp, _i64, C.c_double, C.c_int, _dp, _ip]),
    ("rchol_gpu_pcg_d", C.c_int, [_vp, _vp, _vp, _vp, _i64, C.c_double, C.c_int, _dp, _ip, _vp]),
    ("rchol_gpu_pcg_batch", C.c_int, [_vp, _vp, _i64, _i64p, _dp, _dp, C.c_double, C.c_int, _dp, _ip]),
    ("rchol_gpu_pcg_batch_d", C.c_int, [_vp, _vp, _i64, _i64p, _vp, _vp, C.c_double, C.c_int, _dp, _ip, _vp]),
    ("rchol_gpu_precond_d", C.c_int, [_vp, _vp, _vp, _i64, _vp]),
    ("rchol_gpu_precond_noalloc_d", C.c_int, [_vp, _vp, _vp, _vp]),
    ("rchol_gpu_trsv_d", C.c_int, [_vp, C.c_int, _vp, _vp, _i64, _vp]),
    ("rchol_gpu_spmv_d", C.c_int, [_vp, _vp, _vp, _i64, _vp]),
    ("rchol_gpu_solve_status", C.c_int, [_vp]),
    ("rchol_gpu_wait_selftest", C.c_int, [C.c_uint32, _vp]),
    ("rchol_gpu_edge_grad_d", C.c_int, [_i64, _vp, _vp, _vp, _vp, _vp, _vp]),
]

_lib = None


def lib():
    """Load the library (once).  Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(
                f"{LIB_PATH} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
                "(there is no CPU fallback)")
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


class RcholError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__(f"[status {status}] {msg}")
        self.status = status


def check(rc):
    if rc != OK:
        msg = lib().rchol_gpu_last_error().decode()
        if rc == ERR_INVALID:
            raise ValueError(msg)
        raise RcholError(rc, msg)


def i64(a):
    return np.ascontiguousarray(a, dtype=np.int64)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def p64(a):
    return a.ctypes.data_as(_i64p)


def pd(a):
    return a.ctypes.data_as(_dp)


class Handle:
    _destroy = None

    def __init__(self, ptr):
        self.ptr = ptr

    def close(self):
        if self.ptr:
            getattr(lib(), self._destroy)(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Tree(Handle):
    """Nested-dissection ordering and separator tree (host)."""

    _destroy = "rchol_gpu_tree_destroy"

    @classmethod
    def build(cls, rowptr, colidx, threads, last_in_root=False, leaf_order="natural"):
        """Nested dissection with ``threads`` leaves; ``last_in_root`` gives the
        Python front end's variant (last vertex in the root separator);
        ``leaf_order`` = "natural" (C++ front end), "nd" (METIS nested
        dissection inside leaves) or "md" (minimum degree inside leaves)."""
        rp, ci = i64(rowptr), i64(colidx)
        flags = (1 if last_in_root else 0) | {"natural": 0, "nd": 2, "md": 4}[leaf_order]
        out = _vp()
        check(lib().rchol_gpu_tree_build_ex(len(rp) - 1, p64(rp), p64(ci), int(threads), flags, C.byref(out)))
        return cls(out)

    @classmethod
    def build_batch(cls, sys_ptr, rowptr, colidx, threads):
        """Block-diagonal matrix of independent systems (rows sys_ptr[s] ..
        sys_ptr[s+1]), each ordered on its own; see rchol_gpu_tree_build_batch."""
        sp, rp, ci = i64(sys_ptr), i64(rowptr), i64(colidx)
        out = _vp()
        check(lib().rchol_gpu_tree_build_batch(len(sp) - 1, p64(sp), len(rp) - 1, p64(rp), p64(ci), int(threads),
                                               C.byref(out)))
        return cls(out)

    @classmethod
    def from_partition(cls, perm, part):
        perm, part = i64(perm), i64(part)
        out = _vp()
        check(lib().rchol_gpu_tree_from_partition(len(perm), p64(perm), p64(part), len(part), C.byref(out)))
        return cls(out)

    @property
    def n(self):
        return lib().rchol_gpu_tree_size(self.ptr)

    def arrays(self):
        n = self.n
        np_ = lib().rchol_gpu_tree_num_parts(self.ptr)
        perm = np.zeros(n, np.int64)
        part = np.zeros(np_, np.int64)
        check(lib().rchol_gpu_tree_get(self.ptr, p64(perm), p64(part)))
        return perm, part


def reorder(rowptr, colidx, val, perm):
    """B = A(perm, perm) on the host through the C ABI (c++/util/util.cpp:16-49)."""
    rp, ci, v, p = i64(rowptr), i64(colidx), f64(val), i64(perm)
    n, nnz = len(rp) - 1, int(rp[-1])
    orp, oci, ov = np.zeros(n + 1, np.int64), np.zeros(nnz, np.int64), np.zeros(nnz)
    check(lib().rchol_gpu_reorder(n, p64(rp), p64(ci), pd(v), p64(p), p64(orp), p64(oci), pd(ov)))
    return orp, oci, ov


class Matrix(Handle):
    """SDDM matrix resident on the GPU (stored as A(p,p) when built with a tree)."""

    _destroy = "rchol_gpu_matrix_destroy"

    @classmethod
    def create(cls, rowptr, colidx, val, tree=None):
        rp, ci, v = i64(rowptr), i64(colidx), f64(val)
        out = _vp()
        check(lib().rchol_gpu_matrix_create(len(rp) - 1, p64(rp), p64(ci), pd(v),
                                            tree.ptr if tree else None, C.byref(out)))
        m = cls(out)
        m.n = len(rp) - 1
        return m

    def set_values(self, val):
        v = f64(val)
        check(lib().rchol_gpu_matrix_set_values(self.ptr, pd(v)))


class Factor(Handle):
    """Factor G resident on the GPU."""

    _destroy = "rchol_gpu_factor_destroy"

    @classmethod
    def compute(cls, A: Matrix, tree, seed=0, precision=PREC_FP64):
        out = _vp()
        check(lib().rchol_gpu_factor(A.ptr, tree.ptr if tree else None, C.c_uint64(seed), int(precision),
                                     C.byref(out)))
        f = cls(out)
        f.n = A.n
        return f

    @classmethod
    def from_host(cls, rowptr, colidx, val, tree=None, precision=PREC_FP64):
        rp, ci, v = i64(rowptr), i64(colidx), f64(val)
        out = _vp()
        check(lib().rchol_gpu_factor_from_host(len(rp) - 1, p64(rp), p64(ci), pd(v),
                                               tree.ptr if tree else None, int(precision), C.byref(out)))
        f = cls(out)
        f.n = len(rp) - 1
        return f

    @property
    def nnz(self):
        return lib().rchol_gpu_factor_nnz(self.ptr)

    def export(self):
        """G as CSR of G^T (rowptr, colidx, val)."""
        n, nnz = self.n, self.nnz
        rp, ci, v = np.zeros(n + 1, np.int64), np.zeros(nnz, np.int64), np.zeros(nnz)
        check(lib().rchol_gpu_factor_export(self.ptr, p64(rp), p64(ci), pd(v)))
        return rp, ci, v

    def pivots(self):
        d = np.zeros(self.n)
        check(lib().rchol_gpu_factor_pivots(self.ptr, pd(d)))
        return d

    def levels(self):
        f, b = _i64(), _i64()
        check(lib().rchol_gpu_factor_levels(self.ptr, C.byref(f), C.byref(b)))
        return f.value, b.value

    def plan_info(self, transpose=False):
        """(stages, pieces, sequential block steps) of the forward or backward solve plan."""
        a, b, c = _i64(), _i64(), _i64()
        check(lib().rchol_gpu_factor_plan_info(self.ptr, int(transpose), C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def tune(self):
        """Times the solves with alternative launch choices on this factor and
        keeps the fastest; returns the preconditioner times before and after
        and the chosen values."""
        b, a = C.c_double(), C.c_double()
        k = (C.c_int * 4)()
        check(lib().rchol_gpu_factor_tune(self.ptr, C.byref(b), C.byref(a), k))
        return {"ms_before": b.value, "ms_after": a.value, "pipe_prefetch": k[0], "pipe_ring": k[1],
                "warp_blocks": k[2], "warp_prefetch": k[3]}

    def setup_times(self):
        """Seconds spent in elimination, assembly of G and the solve plan."""
        e, a, p = C.c_double(), C.c_double(), C.c_double()
        check(lib().rchol_gpu_factor_setup_times(self.ptr, C.byref(e), C.byref(a), C.byref(p)))
        return {"eliminate": e.value, "assemble": a.value, "plan": p.value}
