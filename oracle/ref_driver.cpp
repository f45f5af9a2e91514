// Thin C wrapper around the UNMODIFIED reference C++ (compiled from its own
// sources by oracle/Makefile into oracle/_ref/librchol_ref.so).  Test
// infrastructure only: the tests use it to pin the oracle restatement
// (oracle/rchol_oracle.cpp) and to generate the golden fixtures in
// tests/golden/.  Nothing in the product links or loads it.
//
// Every entry point copies its outputs into malloc'd arrays that the caller
// releases with ref_free().  The reference prints progress to std::cout; the
// wrapper silences it for the duration of each call.  Factorizations run on a
// freshly created thread so that the reference's thread_local sampler
// (rchol_lap.cpp:685) starts from the fixed seed on every call.

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <thread>
#include <vector>

#include "sparse.hpp"
#include "rchol.hpp"
#include "rchol_parallel.hpp"
#include "find_separator.hpp"
#include "util.hpp"
#include "laplace_3d.hpp"
#include "pcg.hpp"

extern "C" unsigned int oracle_ref_seed = 0;

// defined (without a header) in c++/rchol/rchol_parallel.cpp:9
SparseCSR remove_diagonal(const SparseCSR &A, std::vector<size_t> &rowPtr,
                          std::vector<size_t> &colIdx, std::vector<double> &val);

namespace {

// Discards everything.  It keeps no put area, so the reference's worker
// threads can write to it concurrently (a stringbuf would race).
struct NullBuf : std::streambuf {
  int overflow(int c) override { return c == EOF ? 0 : c; }
};

struct Quiet {
  NullBuf sink;
  std::streambuf *old;
  Quiet() : old(std::cout.rdbuf(&sink)) {}
  ~Quiet() { std::cout.rdbuf(old); }
};

template <typename T>
T *dup(const T *src, size_t n) {
  T *dst = static_cast<T *>(std::malloc(n ? n * sizeof(T) : sizeof(T)));
  if (n) std::memcpy(dst, src, n * sizeof(T));
  return dst;
}

SparseCSR make_csr(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v) {
  std::vector<size_t> r(rp, rp + n + 1);
  std::vector<size_t> c(ci, ci + rp[n]);
  std::vector<double> x(v, v + rp[n]);
  return SparseCSR(r, c, x, true);
}

void export_csr(const SparseCSR &A, uint64_t **rp, uint64_t **ci, double **v) {
  size_t nnz = A.rowPtr[A.N];
  *rp = dup<uint64_t>(reinterpret_cast<const uint64_t *>(A.rowPtr), A.N + 1);
  *ci = dup<uint64_t>(reinterpret_cast<const uint64_t *>(A.colIdx), nnz);
  *v = dup<double>(A.val, nnz);
}

thread_local std::string g_err;

}  // namespace

extern "C" {

const char *ref_last_error() { return g_err.c_str(); }

void ref_free(void *p) { std::free(p); }

// c++/util/laplace_3d.hpp:8 through c++/util/util.cpp:6
int ref_laplace_3d(int n, int64_t *N, uint64_t **rp, uint64_t **ci, double **v) {
  SparseCSR A = laplace_3d(n);
  A.ownMemory = true;
  *N = (int64_t)A.N;
  export_csr(A, rp, ci, v);
  return 0;
}

// triu_csr + convert_to_laplace + change_to_positive_edge, exactly as
// c++/rchol/rchol.cpp:10-24 chains them.
int ref_extend(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v,
               uint64_t **orp, uint64_t **oci, double **ov) {
  std::vector<size_t> rowPtr(rp, rp + n + 1), colIdx(ci, ci + rp[n]);
  std::vector<double> val(v, v + rp[n]);
  std::vector<size_t> rowPtrU, colIdxU, rowPtrL, colIdxL;
  std::vector<double> valU, valL;
  triu_csr(rowPtr, colIdx, val, rowPtrU, colIdxU, valU);
  convert_to_laplace(rowPtrU, colIdxU, valU, rowPtrL, colIdxL, valL, rowPtr, colIdx, val);
  change_to_positive_edge(valL);
  *orp = dup<uint64_t>(reinterpret_cast<const uint64_t *>(rowPtrL.data()), rowPtrL.size());
  *oci = dup<uint64_t>(reinterpret_cast<const uint64_t *>(colIdxL.data()), colIdxL.size());
  *ov = dup<double>(valL.data(), valL.size());
  return 0;
}

// c++/rchol/rchol_parallel.cpp:37-70: remove_diagonal, find_separator and
// the result_idx prefix (last entry +1 for the ground vertex).
int ref_order(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v,
              int threads, uint64_t **perm, uint64_t **ridx, int64_t *nridx) {
  try {
    Quiet q;
    SparseCSR A = make_csr(n, rp, ci, v);
    std::vector<size_t> r0, c0;
    std::vector<double> v0;
    SparseCSR nd = remove_diagonal(A, r0, c0, v0);
    Separator_info s = find_separator(nd, 1, (size_t)(std::log2(threads) + 1));
    std::vector<size_t> ri{0};
    for (size_t i = 0; i < s.val->size(); ++i) ri.push_back(s.val->at(i) + ri.back());
    ri.back()++;
    *perm = dup<uint64_t>(reinterpret_cast<const uint64_t *>(s.p->data()), s.p->size());
    *ridx = dup<uint64_t>(reinterpret_cast<const uint64_t *>(ri.data()), ri.size());
    *nridx = (int64_t)ri.size();
    delete s.p;
    delete s.val;
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// c++/util/util.cpp:16-49
int ref_reorder(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v,
                const uint64_t *perm, uint64_t **orp, uint64_t **oci, double **ov) {
  SparseCSR A = make_csr(n, rp, ci, v);
  std::vector<size_t> P(perm, perm + n);
  SparseCSR B;
  reorder(A, P, B);
  B.ownMemory = true;
  export_csr(B, orp, oci, ov);
  return 0;
}

// c++/rchol/rchol.cpp:7 (threads == 0) or c++/rchol/rchol_parallel.cpp:37.
// G comes back as the reference returns it: CSR of G^T, diagonal first.
int ref_rchol(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v,
              int threads, unsigned int seed, uint64_t **grp, uint64_t **gci,
              double **gv, uint64_t **perm) {
  int rc = 0;
  std::thread worker([&]() {
    try {
      Quiet q;
      oracle_ref_seed = seed;
      SparseCSR A = make_csr(n, rp, ci, v);
      SparseCSR G;
      std::vector<size_t> P;
      if (threads == 0) {
        rchol(A, G);
        for (int64_t i = 0; i < n; ++i) P.push_back((size_t)i);
      } else {
        rchol(A, G, P, threads);
      }
      export_csr(G, grp, gci, gv);
      *perm = dup<uint64_t>(reinterpret_cast<const uint64_t *>(P.data()), P.size());
      delete[] G.rowPtr;
      delete[] G.colIdx;
      delete[] G.val;
    } catch (const std::exception &e) {
      g_err = e.what();
      rc = 1;
    }
  });
  worker.join();
  return rc;
}

// c++/util/pcg.cpp:14 (the constructor runs the whole solve)
int ref_pcg(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v,
            const double *b, double tol, int maxit, const uint64_t *grp,
            const uint64_t *gci, const double *gv, double *x_out, double *relres,
            int *itr) {
  SparseCSR A = make_csr(n, rp, ci, v);
  SparseCSR G = make_csr(n, grp, gci, gv);
  std::vector<double> bb(b, b + n), x;
  pcg(A, bb, tol, maxit, G, x, *relres, *itr);
  std::memcpy(x_out, x.data(), n * sizeof(double));
  return 0;
}

}  // extern "C"
