// rchol_gb300.hpp -- drop-in C++ front end with the reference's entry points,
// implemented over the C ABI of rchol_gpu.h (link with -lrchol_gb300).
//
//   SparseCSR                        c++/sparse.hpp:10-31 (same fields)
//   laplace_3d(n)                    c++/util/util.cpp:6-12
//   reorder(A, P, B), reorder(x,p,y) c++/util/util.cpp:52-58, util.hpp:147-155
//   rchol(A, G)                      c++/rchol/rchol.hpp:6
//   rchol(A, G, perm, threads)       c++/rchol/rchol_parallel.hpp:6
//   pcg(A, b, tol, maxit, G, x, relres, itr)   c++/util/pcg.hpp:15-16
//
// Differences that a caller can observe:
//  * G owns its memory (ownMemory = true); the reference leaks it.
//  * SparseCSR has move semantics and a deep-copying assignment.
//  * Errors the reference reports with std::invalid_argument still throw
//    std::invalid_argument; GPU failures throw std::runtime_error.
//  * rchol() keeps the factor resident on the GPU; a later pcg() with the same
//    G reuses it instead of uploading G again.
#ifndef RCHOL_GB300_HPP
#define RCHOL_GB300_HPP

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "rchol_gpu.h"

class SparseCSR {
 public:
  SparseCSR() : N(0), rowPtr(nullptr), colIdx(nullptr), val(nullptr), ownMemory(false) {}
  SparseCSR(const std::vector<size_t> &r, const std::vector<size_t> &c, const std::vector<double> &v,
            bool mem = true)
      : SparseCSR() {
    init(r, c, v, mem);
  }
  SparseCSR(const SparseCSR &A) : SparseCSR() { copy_from(A); }
  SparseCSR(SparseCSR &&A) noexcept : SparseCSR() { swap(A); }
  SparseCSR &operator=(const SparseCSR &A) {
    if (this != &A) {
      release();
      copy_from(A);
    }
    return *this;
  }
  SparseCSR &operator=(SparseCSR &&A) noexcept {
    if (this != &A) {
      release();
      swap(A);
    }
    return *this;
  }
  ~SparseCSR() { release(); }

  void init(const std::vector<size_t> &r, const std::vector<size_t> &c, const std::vector<double> &v,
            bool mem = true) {
    release();
    N = r.size() - 1;
    rowPtr = new size_t[N + 1];
    colIdx = new size_t[r[N]];
    val = new double[r[N]];
    std::copy(r.begin(), r.end(), rowPtr);
    std::copy(c.begin(), c.begin() + r[N], colIdx);
    std::copy(v.begin(), v.begin() + r[N], val);
    ownMemory = mem;
  }
  size_t size() const { return N; }
  size_t nnz() const { return rowPtr ? rowPtr[N] : 0; }

  size_t N;
  size_t *rowPtr;
  size_t *colIdx;
  double *val;
  bool ownMemory;

 private:
  void copy_from(const SparseCSR &A) {
    N = A.N;
    if (!A.rowPtr) return;
    rowPtr = new size_t[N + 1];
    colIdx = new size_t[A.nnz()];
    val = new double[A.nnz()];
    std::copy(A.rowPtr, A.rowPtr + N + 1, rowPtr);
    std::copy(A.colIdx, A.colIdx + A.nnz(), colIdx);
    std::copy(A.val, A.val + A.nnz(), val);
    ownMemory = true;
  }
  void swap(SparseCSR &A) noexcept {
    std::swap(N, A.N);
    std::swap(rowPtr, A.rowPtr);
    std::swap(colIdx, A.colIdx);
    std::swap(val, A.val);
    std::swap(ownMemory, A.ownMemory);
  }
  void release() {
    if (ownMemory) {
      delete[] rowPtr;
      delete[] colIdx;
      delete[] val;
    }
    N = 0;
    rowPtr = colIdx = nullptr;
    val = nullptr;
    ownMemory = false;
  }
};

namespace rchol_gb300_detail {

inline void check(int rc) {
  if (rc == RCHOL_OK) return;
  std::string msg = rchol_gpu_last_error();
  if (rc == RCHOL_ERR_INVALID) throw std::invalid_argument(msg);
  throw std::runtime_error(msg);
}

inline const int64_t *i64(const size_t *p) { return reinterpret_cast<const int64_t *>(p); }
static_assert(sizeof(size_t) == sizeof(int64_t), "64-bit size_t expected");

// Factors created by rchol(), kept on the GPU for pcg() with the same G.
struct Resident {
  const double *key;
  size_t n, nnz;
  double first, last;
  std::shared_ptr<rchol_factor_s> factor;
};

inline std::vector<Resident> &resident() {
  static std::vector<Resident> r;
  return r;
}

inline void remember(const SparseCSR &G, rchol_factor_t F) {
  auto &r = resident();
  if (r.size() >= 4) r.erase(r.begin());
  r.push_back(Resident{G.val, G.N, G.nnz(), G.val[0], G.val[G.nnz() - 1],
                       std::shared_ptr<rchol_factor_s>(F, rchol_gpu_factor_destroy)});
}

inline std::shared_ptr<rchol_factor_s> lookup(const SparseCSR &G) {
  for (auto &e : resident())
    if (e.key == G.val && e.n == G.N && e.nnz == G.nnz() && e.first == G.val[0] &&
        e.last == G.val[G.nnz() - 1])
      return e.factor;
  return nullptr;
}

inline void factor_to_csr(rchol_factor_t F, size_t n, SparseCSR &G) {
  std::vector<size_t> rp(n + 1), ci((size_t)rchol_gpu_factor_nnz(F));
  std::vector<double> v(ci.size());
  check(rchol_gpu_factor_export(F, reinterpret_cast<int64_t *>(rp.data()),
                                reinterpret_cast<int64_t *>(ci.data()), v.data()));
  G.init(rp, ci, v, true);
}

inline void factor(const SparseCSR &A, SparseCSR &G, std::vector<size_t> *perm, int threads) {
  rchol_tree_t tree = nullptr;
  check(rchol_gpu_tree_build((int64_t)A.N, i64(A.rowPtr), i64(A.colIdx), threads, &tree));
  std::unique_ptr<rchol_tree_s, void (*)(rchol_tree_t)> tg(tree, rchol_gpu_tree_destroy);
  if (perm) {
    std::vector<int64_t> p(A.N), part((size_t)rchol_gpu_tree_num_parts(tree));
    check(rchol_gpu_tree_get(tree, p.data(), part.data()));
    perm->insert(perm->end(), p.begin(), p.end());  // appends, as the reference does
  }
  rchol_matrix_t M = nullptr;
  check(rchol_gpu_matrix_create((int64_t)A.N, i64(A.rowPtr), i64(A.colIdx), A.val, tree, &M));
  std::unique_ptr<rchol_matrix_s, void (*)(rchol_matrix_t)> mg(M, rchol_gpu_matrix_destroy);
  rchol_factor_t F = nullptr;
  check(rchol_gpu_factor(M, tree, 0, RCHOL_PREC_FP64, &F));
  try {
    factor_to_csr(F, A.N, G);
  } catch (...) {
    rchol_gpu_factor_destroy(F);
    throw;
  }
  remember(G, F);
}

}  // namespace rchol_gb300_detail

// c++/util/util.cpp:6-12 (7-point Dirichlet Laplacian on an n^3 grid).
inline SparseCSR laplace_3d(int n) {
  size_t N = (size_t)n * n * n, n2 = (size_t)n * n;
  std::vector<size_t> rp{0}, ci;
  std::vector<double> v;
  rp.reserve(N + 1);
  ci.reserve(7 * N);
  v.reserve(7 * N);
  for (size_t i = 0; i < (size_t)n; i++)
    for (size_t j = 0; j < (size_t)n; j++)
      for (size_t k = 0; k < (size_t)n; k++) {
        size_t id = k + j * n + i * n2;
        if (i > 0) { ci.push_back(id - n2); v.push_back(-1); }
        if (j > 0) { ci.push_back(id - n); v.push_back(-1); }
        if (k > 0) { ci.push_back(id - 1); v.push_back(-1); }
        ci.push_back(id); v.push_back(6);
        if (k + 1 < (size_t)n) { ci.push_back(id + 1); v.push_back(-1); }
        if (j + 1 < (size_t)n) { ci.push_back(id + n); v.push_back(-1); }
        if (i + 1 < (size_t)n) { ci.push_back(id + n2); v.push_back(-1); }
        rp.push_back(ci.size());
      }
  return SparseCSR(rp, ci, v, true);
}

// c++/util/util.cpp:52-58
inline void reorder(const SparseCSR &A, const std::vector<size_t> &P, SparseCSR &B) {
  std::vector<size_t> rp(A.N + 1), ci(A.nnz());
  std::vector<double> v(A.nnz());
  rchol_gb300_detail::check(rchol_gpu_reorder(
      (int64_t)A.N, rchol_gb300_detail::i64(A.rowPtr), rchol_gb300_detail::i64(A.colIdx), A.val,
      rchol_gb300_detail::i64(P.data()), reinterpret_cast<int64_t *>(rp.data()),
      reinterpret_cast<int64_t *>(ci.data()), v.data()));
  B.init(rp, ci, v, true);
}

// c++/util/util.hpp:147-164
template <typename T>
void reorder(std::vector<T> &x, std::vector<size_t> &p, std::vector<T> &xp) {
  xp.reserve(p.size());
  for (size_t i = 0; i < x.size(); i++) xp.push_back(x[p[i]]);
}

// c++/rchol/rchol.cpp:7-28: natural order, one subdomain.
inline void rchol(const SparseCSR &A, SparseCSR &G) { rchol_gb300_detail::factor(A, G, nullptr, 1); }

// c++/rchol/rchol_parallel.cpp:37-92: nested dissection with `threads` leaf
// subdomains (a power of two); appends the permutation to `permutation`.
inline void rchol(const SparseCSR &A, SparseCSR &G, std::vector<size_t> &permutation, int threads) {
  if (threads <= 0) throw std::invalid_argument("thread number should be positive");
  if ((threads & (threads - 1)) != 0) throw std::invalid_argument("thread number should be a power of 2");
  rchol_gb300_detail::factor(A, G, &permutation, threads);
}

// c++/util/pcg.hpp:13-26: the constructor runs the whole solve.
class pcg {
 public:
  pcg(const SparseCSR &A, const std::vector<double> &b, double tol, int maxit, const SparseCSR &G,
      std::vector<double> &x, double &relres, int &itr) {
    using namespace rchol_gb300_detail;
    std::shared_ptr<rchol_factor_s> F = lookup(G);
    if (!F) {
      rchol_factor_t f = nullptr;
      check(rchol_gpu_factor_from_host((int64_t)G.N, i64(G.rowPtr), i64(G.colIdx), G.val, nullptr,
                                       RCHOL_PREC_FP64, &f));
      F.reset(f, rchol_gpu_factor_destroy);
    }
    rchol_matrix_t M = nullptr;
    check(rchol_gpu_matrix_create((int64_t)A.N, i64(A.rowPtr), i64(A.colIdx), A.val, nullptr, &M));
    std::unique_ptr<rchol_matrix_s, void (*)(rchol_matrix_t)> mg(M, rchol_gpu_matrix_destroy);
    x.assign(A.N, 0.0);
    check(rchol_gpu_pcg(M, F.get(), b.data(), x.data(), 1, tol, maxit, &relres, &itr));
  }
};

#endif  // RCHOL_GB300_HPP
