/* Serial stand-in for the handful of MKL sparse-BLAS / CBLAS calls used by
 * the reference's c++/util/pcg.cpp, written from MKL's documented semantics:
 *   mkl_sparse_d_create_csr  wraps 0-based CSR arrays (no copy)
 *   mkl_sparse_d_mv          y = alpha*op(A)*x + beta*y  (op = N only)
 *   mkl_sparse_d_trsv        solves op(A)*y = alpha*x for a triangular A
 *   cblas_d{nrm2,dot,copy,scal,axpy} with unit stride.
 * The reference stores U = G^T (upper, non-unit diagonal first in each row);
 * op=T is a forward substitution with U^T, op=N a backward one with U.
 * Test infrastructure only: it lets the unmodified reference compile. */
#pragma once
#include <cmath>
#include <cstring>
#ifndef MKL_INT
#define MKL_INT long long
#endif

enum sparse_status_t { SPARSE_STATUS_SUCCESS = 0 };
enum sparse_index_base_t { SPARSE_INDEX_BASE_ZERO = 0, SPARSE_INDEX_BASE_ONE = 1 };
enum sparse_operation_t {
  SPARSE_OPERATION_NON_TRANSPOSE = 10,
  SPARSE_OPERATION_TRANSPOSE = 11,
  SPARSE_OPERATION_CONJUGATE_TRANSPOSE = 12
};
enum sparse_matrix_type_t {
  SPARSE_MATRIX_TYPE_GENERAL = 20,
  SPARSE_MATRIX_TYPE_SYMMETRIC = 21,
  SPARSE_MATRIX_TYPE_HERMITIAN = 22,
  SPARSE_MATRIX_TYPE_TRIANGULAR = 23
};
enum sparse_fill_mode_t { SPARSE_FILL_MODE_LOWER = 40, SPARSE_FILL_MODE_UPPER = 41 };
enum sparse_diag_type_t { SPARSE_DIAG_NON_UNIT = 50, SPARSE_DIAG_UNIT = 51 };

struct matrix_descr {
  sparse_matrix_type_t type;
  sparse_fill_mode_t mode;
  sparse_diag_type_t diag;
};

struct oracle_shim_csr {
  long long rows;
  MKL_INT *row_begin;
  MKL_INT *row_end;
  MKL_INT *cols;
  double *vals;
};
typedef oracle_shim_csr *sparse_matrix_t;

inline sparse_status_t mkl_sparse_d_create_csr(sparse_matrix_t *A, sparse_index_base_t,
                                               MKL_INT rows, MKL_INT, MKL_INT *rb,
                                               MKL_INT *re, MKL_INT *ci, double *v) {
  *A = new oracle_shim_csr{(long long)rows, rb, re, ci, v};
  return SPARSE_STATUS_SUCCESS;
}

inline sparse_status_t mkl_sparse_destroy(sparse_matrix_t A) {
  delete A;
  return SPARSE_STATUS_SUCCESS;
}

inline sparse_status_t mkl_sparse_d_mv(sparse_operation_t, double alpha, sparse_matrix_t A,
                                       matrix_descr, const double *x, double beta,
                                       double *y) {
  for (long long r = 0; r < A->rows; ++r) {
    double acc = 0.0;
    for (long long k = (long long)A->row_begin[r]; k < (long long)A->row_end[r]; ++k)
      acc += A->vals[k] * x[A->cols[k]];
    y[r] = (beta == 0.0) ? alpha * acc : alpha * acc + beta * y[r];
  }
  return SPARSE_STATUS_SUCCESS;
}

inline sparse_status_t mkl_sparse_d_trsv(sparse_operation_t op, double alpha,
                                         sparse_matrix_t A, matrix_descr,
                                         const double *x, double *y) {
  const long long n = A->rows;
  if (op == SPARSE_OPERATION_TRANSPOSE) {
    /* U^T y = alpha x : column sweep of U in increasing row order */
    for (long long r = 0; r < n; ++r) y[r] = alpha * x[r];
    for (long long r = 0; r < n; ++r) {
      double diag = 0.0;
      for (long long k = (long long)A->row_begin[r]; k < (long long)A->row_end[r]; ++k)
        if ((long long)A->cols[k] == r) diag = A->vals[k];
      y[r] /= diag;
      for (long long k = (long long)A->row_begin[r]; k < (long long)A->row_end[r]; ++k)
        if ((long long)A->cols[k] > r) y[A->cols[k]] -= A->vals[k] * y[r];
    }
  } else {
    /* U y = alpha x : backward substitution, signed loop index */
    for (long long r = n - 1; r >= 0; --r) {
      double acc = alpha * x[r], diag = 0.0;
      for (long long k = (long long)A->row_begin[r]; k < (long long)A->row_end[r]; ++k) {
        long long c = (long long)A->cols[k];
        if (c == r) diag = A->vals[k];
        else if (c > r) acc -= A->vals[k] * y[c];
      }
      y[r] = acc / diag;
    }
  }
  return SPARSE_STATUS_SUCCESS;
}

inline double cblas_dnrm2(MKL_INT n, const double *x, MKL_INT) {
  double s = 0.0;
  for (long long i = 0; i < (long long)n; ++i) s += x[i] * x[i];
  return std::sqrt(s);
}
inline double cblas_ddot(MKL_INT n, const double *x, MKL_INT, const double *y, MKL_INT) {
  double s = 0.0;
  for (long long i = 0; i < (long long)n; ++i) s += x[i] * y[i];
  return s;
}
inline void cblas_dcopy(MKL_INT n, const double *x, MKL_INT, double *y, MKL_INT) {
  std::memcpy(y, x, (size_t)n * sizeof(double));
}
inline void cblas_dscal(MKL_INT n, double a, double *x, MKL_INT) {
  for (long long i = 0; i < (long long)n; ++i) x[i] *= a;
}
inline void cblas_daxpy(MKL_INT n, double a, const double *x, MKL_INT, double *y, MKL_INT) {
  for (long long i = 0; i < (long long)n; ++i) y[i] += a * x[i];
}
