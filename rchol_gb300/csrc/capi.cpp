// C ABI of include/rchol_gpu.h.  Every entry point converts exceptions into
// a status code and a thread-local message.

#include <algorithm>
#include <chrono>
#include <atomic>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>

#include "common.hpp"
#include "host.hpp"
#include "plan.hpp"
#include "tree_infer.hpp"

namespace rchol {

namespace {
thread_local std::string g_last_error;
std::atomic<int64_t> g_launches{0};
std::atomic<uint64_t> g_matrix_uid{0};
}  // namespace

void set_last_error(const std::string &msg) { g_last_error = msg; }
void note_launch(int64_t count) { g_launches.fetch_add(count, std::memory_order_relaxed); }

void trsv(const rchol_factor_s &F, bool upper, const double *in, double *out, int k, cudaStream_t s);
void precond(const rchol_factor_s &F, const double *r, double *z, int k, cudaStream_t s);
void spmv_public(const rchol_matrix_s &A, const double *x, double *y, int k, cudaStream_t s);
void pcg_device(const rchol_matrix_s &A, const rchol_factor_s &F, const double *b, double *x, int k,
                double tol, int maxit, double *relres, int *itr, cudaStream_t s);
void pcg_host(const rchol_matrix_s &A, const rchol_factor_s &F, const double *b, double *x, int k,
              double tol, int maxit, double *relres, int *itr);
int64_t plan_levels(const rchol_factor_s &F, bool upper);
void pcg_batch_device(const rchol_matrix_s &A, const rchol_factor_s &F, int64_t nseg, const int64_t *seg,
                      const double *b, double *x, double tol, int maxit, double *relres, int *itr,
                      cudaStream_t s);
void pcg_batch_host(const rchol_matrix_s &A, const rchol_factor_s &F, int64_t nseg, const int64_t *seg,
                    const double *b, double *x, double tol, int maxit, double *relres, int *itr);
uint32_t take_solve_status(cudaStream_t s);
void check_solve_status(cudaStream_t s);
void wait_selftest(uint32_t polls, cudaStream_t s);
void edge_grad(int64_t m, const int64_t *ei, const int64_t *ej, const double *lam, const double *x, double *g,
               cudaStream_t s);
void precond_noalloc(const rchol_factor_s &F, const double *r, double *z, cudaStream_t s);

}  // namespace rchol

using namespace rchol;

#define API_BEGIN try {
#define API_END                          \
  return RCHOL_OK;                       \
  }                                      \
  catch (const Error &e) {               \
    set_last_error(e.what());            \
    return e.status;                     \
  }                                      \
  catch (const std::bad_alloc &) {       \
    set_last_error("host allocation failed"); \
    return RCHOL_ERR_NOMEM;              \
  }                                      \
  catch (const std::exception &e) {      \
    set_last_error(e.what());            \
    return RCHOL_ERR_INTERNAL;           \
  }

static cudaStream_t as_stream(void *s) { return reinterpret_cast<cudaStream_t>(s); }

extern "C" {

const char *rchol_gpu_last_error(void) { return g_last_error.c_str(); }
const char *rchol_gpu_version(void) { return "rchol_gb300 0.1 (sm_103a)"; }
int64_t rchol_gpu_launch_count(void) { return g_launches.load(); }

// ---- ordering ---------------------------------------------------------------

int rchol_gpu_tree_build(int64_t n, const int64_t *row_ptr, const int64_t *col_idx, int threads,
                         rchol_tree_t *out) {
  API_BEGIN
  RCHOL_CHECK_ARG(out, "null output handle");
  *out = nullptr;
  *out = build_tree(n, row_ptr, col_idx, threads);
  API_END
}

int rchol_gpu_tree_build_ex(int64_t n, const int64_t *row_ptr, const int64_t *col_idx, int threads, int flags,
                            rchol_tree_t *out) {
  API_BEGIN
  RCHOL_CHECK_ARG(out, "null output handle");
  RCHOL_CHECK_ARG((flags & ~(RCHOL_ORDER_LAST_IN_ROOT | RCHOL_ORDER_LEAF_ND | RCHOL_ORDER_LEAF_MD)) == 0,
                  "unknown ordering flags");
  RCHOL_CHECK_ARG(!((flags & RCHOL_ORDER_LEAF_ND) && (flags & RCHOL_ORDER_LEAF_MD)), "choose one leaf ordering");
  *out = nullptr;
  const int leaf = (flags & RCHOL_ORDER_LEAF_ND) ? RCHOL_LEAF_ND : (flags & RCHOL_ORDER_LEAF_MD) ? RCHOL_LEAF_MD
                                                                                                   : RCHOL_LEAF_NATURAL;
  *out = build_tree(n, row_ptr, col_idx, threads, (flags & RCHOL_ORDER_LAST_IN_ROOT) != 0, leaf);
  API_END
}

int rchol_gpu_tree_build_batch(int64_t nsys, const int64_t *sys_ptr, int64_t n, const int64_t *row_ptr,
                               const int64_t *col_idx, int threads, rchol_tree_t *out) {
  API_BEGIN
  RCHOL_CHECK_ARG(out, "null output handle");
  *out = nullptr;
  *out = build_tree_batch(nsys, sys_ptr, n, row_ptr, col_idx, threads);
  API_END
}

int rchol_gpu_tree_from_partition(int64_t n, const int64_t *perm, const int64_t *part,
                                  int64_t nparts, rchol_tree_t *out) {
  API_BEGIN
  RCHOL_CHECK_ARG(out, "null output handle");
  *out = nullptr;
  *out = tree_from_partition(n, perm, part, nparts);
  API_END
}

int64_t rchol_gpu_tree_size(rchol_tree_t t) { return t ? t->n : -1; }
int64_t rchol_gpu_tree_num_parts(rchol_tree_t t) { return t ? (int64_t)t->part.size() : -1; }

int rchol_gpu_tree_get(rchol_tree_t t, int64_t *perm, int64_t *part) {
  API_BEGIN
  RCHOL_CHECK_ARG(t, "null tree");
  if (perm) std::memcpy(perm, t->perm.data(), t->perm.size() * sizeof(int64_t));
  if (part) std::memcpy(part, t->part.data(), t->part.size() * sizeof(int64_t));
  API_END
}

void rchol_gpu_tree_destroy(rchol_tree_t t) { delete t; }

int rchol_gpu_reorder(int64_t n, const int64_t *row_ptr, const int64_t *col_idx, const double *val,
                      const int64_t *perm, int64_t *out_row_ptr, int64_t *out_col_idx,
                      double *out_val) {
  API_BEGIN
  RCHOL_CHECK_ARG(val && perm && out_row_ptr && out_col_idx && out_val, "null argument");
  validate_csr(n, row_ptr, col_idx);
  std::vector<char> seen(n, 0);
  for (int64_t i = 0; i < n; ++i) {
    RCHOL_CHECK_ARG(perm[i] >= 0 && perm[i] < n && !seen[perm[i]], "perm is not a permutation");
    seen[perm[i]] = 1;
  }
  HostCsr B = reorder(n, row_ptr, col_idx, val, std::vector<int64_t>(perm, perm + n));
  std::memcpy(out_row_ptr, B.rp.data(), (n + 1) * sizeof(int64_t));
  std::memcpy(out_col_idx, B.ci.data(), B.ci.size() * sizeof(int64_t));
  std::memcpy(out_val, B.v.data(), B.v.size() * sizeof(double));
  API_END
}

// ---- matrices ---------------------------------------------------------------

int rchol_gpu_matrix_create(int64_t n, const int64_t *row_ptr, const int64_t *col_idx,
                            const double *val, rchol_tree_t tree, rchol_matrix_t *out) {
  API_BEGIN
  RCHOL_CHECK_ARG(out && val, "null argument");
  *out = nullptr;
  validate_csr(n, row_ptr, col_idx);
  RCHOL_CHECK_ARG(!tree || tree->n == n, "tree and matrix sizes differ");
  std::unique_ptr<rchol_matrix_s> A(new rchol_matrix_s());
  A->uid = ++g_matrix_uid;
  A->n = n;
  A->nnz = row_ptr[n];
  if (tree) {
    A->permuted = true;
    A->perm = tree->perm;
    A->host = reorder(n, row_ptr, col_idx, val, tree->perm, &A->srcpos);
  } else {
    A->host.n = n;
    A->host.rp.assign(row_ptr, row_ptr + n + 1);
    A->host.ci.assign(col_idx, col_idx + A->nnz);
    A->host.v.assign(val, val + A->nnz);
  }
  std::vector<int32_t> ci32(A->nnz);
  parallel_for(A->nnz, [&](int64_t a, int64_t b) {
    for (int64_t i = a; i < b; ++i) ci32[i] = (int32_t)A->host.ci[i];
  }, 1 << 20);
  A->rp.upload(A->host.rp.data(), n + 1);
  A->ci.upload(ci32.data(), A->nnz);
  A->v.upload(A->host.v.data(), A->nnz);
  RCHOL_CUDA(cudaDeviceSynchronize());
  build_sell(*A);
  *out = A.release();
  API_END
}

int64_t rchol_gpu_matrix_size(rchol_matrix_t A) { return A ? A->n : -1; }
int64_t rchol_gpu_matrix_nnz(rchol_matrix_t A) { return A ? A->nnz : -1; }

int rchol_gpu_matrix_set_values(rchol_matrix_t A, const double *val) {
  API_BEGIN
  RCHOL_CHECK_ARG(A && val, "null argument");
  if (A->permuted) {
    for (int64_t q = 0; q < A->nnz; ++q) A->host.v[q] = val[A->srcpos[q]];
  } else {
    A->host.v.assign(val, val + A->nnz);
  }
  A->v.upload(A->host.v.data(), A->nnz);
  RCHOL_CUDA(cudaDeviceSynchronize());
  build_sell(*A);
  API_END
}

void rchol_gpu_matrix_destroy(rchol_matrix_t A) { delete A; }

// ---- factorization -------------------------------------------------------------

int rchol_gpu_factor(rchol_matrix_t A, rchol_tree_t tree, uint64_t seed, int precision,
                     rchol_factor_t *out) {
  API_BEGIN
  RCHOL_CHECK_ARG(A && out, "null argument");
  *out = nullptr;
  RCHOL_CHECK_ARG(precision == RCHOL_PREC_FP64 || precision == RCHOL_PREC_FP32, "bad precision");
  RCHOL_CHECK_ARG(!tree || tree->n == A->n, "tree and matrix sizes differ");
  RCHOL_CHECK_ARG(!tree || A->permuted, "matrix was created without the tree");
  RCHOL_CHECK_ARG(tree || !A->permuted, "matrix was created with a tree; pass it");
  HostCsr ext = extend_laplacian(A->host);
  std::unique_ptr<rchol_factor_s> F(new rchol_factor_s());
  F->precision = precision;
  F->nodes = tree ? tree->nodes : trivial_nodes(A->n);
  cudaStream_t s = 0;
  const auto t0 = std::chrono::steady_clock::now();
  gpu_factor(ext, F->nodes, seed, *F, s);
  RCHOL_CUDA(cudaStreamSynchronize(s));
  F->t_eliminate = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  finish_factor(*F, s);
  *out = F.release();
  API_END
}

int rchol_gpu_factor_from_host(int64_t n, const int64_t *row_ptr, const int64_t *col_idx,
                               const double *val, rchol_tree_t tree, int precision,
                               rchol_factor_t *out) {
  API_BEGIN
  RCHOL_CHECK_ARG(out && val, "null argument");
  *out = nullptr;
  RCHOL_CHECK_ARG(precision == RCHOL_PREC_FP64 || precision == RCHOL_PREC_FP32, "bad precision");
  validate_csr(n, row_ptr, col_idx);
  for (int64_t i = 0; i < n; ++i)
    RCHOL_CHECK_ARG(row_ptr[i + 1] > row_ptr[i] && col_idx[row_ptr[i]] == i && val[row_ptr[i]] != 0.0,
                    "G^T must be upper triangular with a nonzero diagonal first in every row");
  RCHOL_CHECK_ARG(!tree || tree->n == n, "tree and factor sizes differ");
  std::unique_ptr<rchol_factor_s> F(new rchol_factor_s());
  F->n = n;
  F->nnz = row_ptr[n];
  F->precision = precision;
  // without a tree (a G made elsewhere, or copied): the tree its nonzero
  // pattern shows, so that independent subtrees are solved in parallel
  F->nodes = tree ? tree->nodes : infer_factor_tree(n, row_ptr, col_idx);
  std::vector<int32_t> ci32(F->nnz);
  for (int64_t i = 0; i < F->nnz; ++i) ci32[i] = (int32_t)col_idx[i];
  cudaStream_t s = 0;
  F->urp.upload(row_ptr, n + 1, s);
  F->uci.upload(ci32.data(), F->nnz, s);
  F->uv.upload(val, F->nnz, s);
  RCHOL_CUDA(cudaStreamSynchronize(s));
  finish_factor(*F, s);
  *out = F.release();
  API_END
}

int64_t rchol_gpu_factor_nnz(rchol_factor_t G) { return G ? G->nnz : -1; }

int rchol_gpu_factor_plan_info(rchol_factor_t G, int transpose, int64_t *stages, int64_t *pieces, int64_t *steps) {
  API_BEGIN
  RCHOL_CHECK_ARG(G && G->plan, "null factor");
  const StreamDir &D = transpose ? G->plan->sbwd : G->plan->sfwd;
  if (stages) *stages = (int64_t)D.stage_ptr.size() - 1;
  if (pieces) *pieces = D.stage_ptr.empty() ? 0 : D.stage_ptr.back();
  if (steps) *steps = D.steps;
  API_END
}

int rchol_gpu_factor_tune(rchol_factor_t G, double *ms_before, double *ms_after, int *knobs) {
  API_BEGIN
  RCHOL_CHECK_ARG(G && G->plan, "null factor");
  std::lock_guard<std::mutex> guard(G->plan->lock);
  const std::pair<double, double> t = tune_solves(*G, *G->plan, 0);
  if (ms_before) *ms_before = t.first;
  if (ms_after) *ms_after = t.second;
  if (knobs) {
    const SolveKnobs &k = G->plan->knobs;
    knobs[0] = k.pipe_pf;
    knobs[1] = k.pipe_ring;
    knobs[2] = k.w2_wpb;
    knobs[3] = k.w2_pf;
  }
  API_END
}

int rchol_gpu_factor_setup_times(rchol_factor_t G, double *eliminate_s, double *assemble_s, double *plan_s) {
  API_BEGIN
  RCHOL_CHECK_ARG(G, "null factor");
  if (eliminate_s) *eliminate_s = G->t_eliminate;
  if (assemble_s) *assemble_s = G->t_assemble;
  if (plan_s) *plan_s = G->t_plan;
  API_END
}
int rchol_gpu_factor_precision(rchol_factor_t G) { return G ? G->precision : -1; }

int rchol_gpu_factor_export(rchol_factor_t G, int64_t *row_ptr, int64_t *col_idx, double *val) {
  API_BEGIN
  RCHOL_CHECK_ARG(G, "null factor");
  if (row_ptr) G->urp.download(row_ptr, G->n + 1);
  if (val) G->uv.download(val, G->nnz);
  if (col_idx) {
    std::vector<int32_t> ci(G->nnz);
    G->uci.download(ci.data(), G->nnz);
    RCHOL_CUDA(cudaDeviceSynchronize());
    for (int64_t i = 0; i < G->nnz; ++i) col_idx[i] = ci[i];
  }
  RCHOL_CUDA(cudaDeviceSynchronize());
  API_END
}

int rchol_gpu_factor_pivots(rchol_factor_t G, double *d) {
  API_BEGIN
  RCHOL_CHECK_ARG(G && d, "null argument");
  RCHOL_CHECK_ARG(G->pivots.n == (size_t)G->n, "factor has no pivots (loaded from host)");
  G->pivots.download(d, G->n);
  RCHOL_CUDA(cudaDeviceSynchronize());
  API_END
}

int rchol_gpu_factor_levels(rchol_factor_t G, int64_t *fwd, int64_t *bwd) {
  API_BEGIN
  RCHOL_CHECK_ARG(G && G->plan, "null factor");
  if (fwd) *fwd = plan_levels(*G, false);
  if (bwd) *bwd = plan_levels(*G, true);
  API_END
}

void rchol_gpu_factor_destroy(rchol_factor_t G) { delete G; }

// ---- solves -------------------------------------------------------------------------

int rchol_gpu_pcg_d(rchol_matrix_t A, rchol_factor_t G, const double *d_b, double *d_x,
                    int64_t nrhs, double tol, int maxit, double *relres, int *itr, void *stream) {
  API_BEGIN
  RCHOL_CHECK_ARG(A && G && d_b && d_x && relres && itr, "null argument");
  RCHOL_CHECK_ARG(A->n == G->n, "matrix and factor sizes differ");
  RCHOL_CHECK_ARG(nrhs >= 1 && nrhs <= 256, "nrhs must be in [1, 256]");
  RCHOL_CHECK_ARG(maxit >= 0, "maxit must be nonnegative");
  pcg_device(*A, *G, d_b, d_x, (int)nrhs, tol, maxit, relres, itr, as_stream(stream));
  check_solve_status(as_stream(stream));
  API_END
}

int rchol_gpu_pcg(rchol_matrix_t A, rchol_factor_t G, const double *b, double *x, int64_t nrhs,
                  double tol, int maxit, double *relres, int *itr) {
  API_BEGIN
  RCHOL_CHECK_ARG(A && G && b && x && relres && itr, "null argument");
  RCHOL_CHECK_ARG(A->n == G->n, "matrix and factor sizes differ");
  RCHOL_CHECK_ARG(nrhs >= 1 && nrhs <= 256, "nrhs must be in [1, 256]");
  pcg_host(*A, *G, b, x, (int)nrhs, tol, maxit, relres, itr);
  check_solve_status(nullptr);
  API_END
}

static void check_systems(rchol_matrix_t A, int64_t nsys, const int64_t *sys_ptr) {
  RCHOL_CHECK_ARG(nsys >= 1 && sys_ptr, "need at least one system");
  RCHOL_CHECK_ARG(sys_ptr[0] == 0 && sys_ptr[nsys] == A->n, "system offsets must run from 0 to n");
  for (int64_t s = 0; s < nsys; ++s)
    RCHOL_CHECK_ARG(sys_ptr[s + 1] > sys_ptr[s], "every system needs at least one row");
}

int rchol_gpu_pcg_batch_d(rchol_matrix_t A, rchol_factor_t G, int64_t nsys, const int64_t *sys_ptr,
                          const double *d_b, double *d_x, double tol, int maxit, double *relres, int *itr,
                          void *stream) {
  API_BEGIN
  RCHOL_CHECK_ARG(A && G && d_b && d_x && relres && itr, "null argument");
  RCHOL_CHECK_ARG(A->n == G->n, "matrix and factor sizes differ");
  RCHOL_CHECK_ARG(maxit >= 0, "maxit must be nonnegative");
  check_systems(A, nsys, sys_ptr);
  pcg_batch_device(*A, *G, nsys, sys_ptr, d_b, d_x, tol, maxit, relres, itr, as_stream(stream));
  check_solve_status(as_stream(stream));
  API_END
}

int rchol_gpu_pcg_batch(rchol_matrix_t A, rchol_factor_t G, int64_t nsys, const int64_t *sys_ptr,
                        const double *b, double *x, double tol, int maxit, double *relres, int *itr) {
  API_BEGIN
  RCHOL_CHECK_ARG(A && G && b && x && relres && itr, "null argument");
  RCHOL_CHECK_ARG(A->n == G->n, "matrix and factor sizes differ");
  RCHOL_CHECK_ARG(maxit >= 0, "maxit must be nonnegative");
  check_systems(A, nsys, sys_ptr);
  pcg_batch_host(*A, *G, nsys, sys_ptr, b, x, tol, maxit, relres, itr);
  check_solve_status(nullptr);
  API_END
}

int rchol_gpu_precond_d(rchol_factor_t G, const double *d_r, double *d_z, int64_t nrhs,
                        void *stream) {
  API_BEGIN
  RCHOL_CHECK_ARG(G && d_r && d_z, "null argument");
  RCHOL_CHECK_ARG(nrhs >= 1 && nrhs <= 256, "nrhs must be in [1, 256]");
  precond(*G, d_r, d_z, (int)nrhs, as_stream(stream));
  API_END
}

int rchol_gpu_precond_noalloc_d(rchol_factor_t G, const double *d_r, double *d_z, void *stream) {
  API_BEGIN
  RCHOL_CHECK_ARG(G && G->plan && d_r && d_z, "null argument");
  precond_noalloc(*G, d_r, d_z, as_stream(stream));
  API_END
}

int rchol_gpu_trsv_d(rchol_factor_t G, int transpose, const double *d_in, double *d_out,
                     int64_t nrhs, void *stream) {
  API_BEGIN
  RCHOL_CHECK_ARG(G && d_in && d_out, "null argument");
  RCHOL_CHECK_ARG(nrhs >= 1 && nrhs <= 256, "nrhs must be in [1, 256]");
  trsv(*G, transpose != 0, d_in, d_out, (int)nrhs, as_stream(stream));
  API_END
}

int rchol_gpu_solve_status(void *stream) {
  API_BEGIN
  check_solve_status(as_stream(stream));
  API_END
}

int rchol_gpu_wait_selftest(uint32_t polls, void *stream) {
  API_BEGIN
  wait_selftest(polls, as_stream(stream));
  check_solve_status(as_stream(stream));
  API_END
}

int rchol_gpu_edge_grad_d(int64_t nedges, const int64_t *d_ei, const int64_t *d_ej, const double *d_lambda,
                          const double *d_x, double *d_grad, void *stream) {
  API_BEGIN
  RCHOL_CHECK_ARG(nedges >= 0, "nedges must be nonnegative");
  RCHOL_CHECK_ARG(nedges == 0 || (d_ei && d_ej && d_lambda && d_x && d_grad), "null argument");
  edge_grad(nedges, d_ei, d_ej, d_lambda, d_x, d_grad, as_stream(stream));
  API_END
}

int rchol_gpu_spmv_d(rchol_matrix_t A, const double *d_x, double *d_y, int64_t nrhs, void *stream) {
  API_BEGIN
  RCHOL_CHECK_ARG(A && d_x && d_y, "null argument");
  RCHOL_CHECK_ARG(nrhs >= 1 && nrhs <= 256, "nrhs must be in [1, 256]");
  spmv_public(*A, d_x, d_y, (int)nrhs, as_stream(stream));
  API_END
}

}  // extern "C"
