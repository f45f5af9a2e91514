// SpMV with A, the transposed copy and FP32 copy of G, the solve plan, and
// the PCG loops of c++/util/pcg.cpp:57-159 on the GPU (one system with k
// right-hand sides, and many independent systems at once).  The triangular
// solves themselves are in trsv.cu.
//
// Several right-hand sides are stored row-major (n x k); every right-hand
// side keeps its own PCG scalars and stopping test.

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <numeric>
#include <vector>

#include "common.hpp"
#include "host.hpp"
#include "plan.hpp"

namespace rchol {

void exclusive_scan_i64(int64_t *d_data, int64_t n, cudaStream_t s);

void destroy_plan(SolvePlan *p) { delete p; }

namespace {

// ---- SpMV ---------------------------------------------------------------------

// y = A x for one right-hand side: LPR lanes per row.
template <int LPR>
__global__ void spmv1_kernel(int64_t n, const int64_t *__restrict__ rp, const int32_t *__restrict__ ci,
                             const double *__restrict__ v, const double *__restrict__ x,
                             double *__restrict__ y) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  int64_t row = t / LPR;
  int sub = (int)(t % LPR);
  double s = 0.0;
  if (row < n)  // no early return: every lane takes part in the shuffles
    for (int64_t q = rp[row] + sub; q < rp[row + 1]; q += LPR) s += v[q] * x[ci[q]];
#pragma unroll
  for (int o = LPR / 2; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o, LPR);
  if (sub == 0 && row < n) y[row] = s;
}

// y = A x for k right-hand sides stored row-major; one warp per row, lanes over k.
__global__ void spmvk_kernel(int64_t n, int k, const int64_t *__restrict__ rp,
                             const int32_t *__restrict__ ci, const double *__restrict__ v,
                             const double *__restrict__ x, double *__restrict__ y) {
  int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= n) return;
  for (int r = lane; r < k; r += 32) {
    double s = 0.0;
    for (int64_t q = rp[row]; q < rp[row + 1]; ++q) s += v[q] * x[(int64_t)ci[q] * k + r];
    y[row * k + r] = s;
  }
}

// y = A x, sliced ELL: one thread per row, each of a warp's loads is one
// contiguous 128/256-byte transaction.
__global__ void __launch_bounds__(256) spmv_sell_kernel(int64_t n, const int64_t *__restrict__ off,
                                                        const int32_t *__restrict__ ci,
                                                        const double *__restrict__ v,
                                                        const double *__restrict__ x, double *__restrict__ y) {
  const int64_t row = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (row >= n) return;
  const int64_t sl = row >> 5;
  const int t = (int)(row & 31);
  const int64_t o0 = off[sl], w = (off[sl + 1] - o0) >> 5;
  double s0 = 0.0, s1 = 0.0;
  int64_t j = 0;
  for (; j + 1 < w; j += 2) {
    s0 += __ldg(&v[o0 + 32 * j + t]) * __ldg(&x[__ldg(&ci[o0 + 32 * j + t])]);
    s1 += __ldg(&v[o0 + 32 * (j + 1) + t]) * __ldg(&x[__ldg(&ci[o0 + 32 * (j + 1) + t])]);
  }
  if (j < w) s0 += __ldg(&v[o0 + 32 * j + t]) * __ldg(&x[__ldg(&ci[o0 + 32 * j + t])]);
  y[row] = s0 + s1;
}

void spmv(const rchol_matrix_s &A, const double *x, double *y, int k, cudaStream_t s) {
  const int64_t n = A.n;
  if (k == 1 && A.sell_off.p) {
    spmv_sell_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, A.sell_off.p, A.sell_ci.p, A.sell_v.p, x, y);
    note_launch();
  } else if (k == 1) {
    int64_t threads = n * 8;
    spmv1_kernel<8><<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(n, A.rp.p, A.ci.p, A.v.p, x, y);
    note_launch();
  } else {
    int64_t threads = n * 32;
    spmvk_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(n, k, A.rp.p, A.ci.p, A.v.p, x, y);
    note_launch();
  }
  RCHOL_CUDA(cudaGetLastError());
}

}  // namespace

void build_sell(rchol_matrix_s &A) {
  const HostCsr &H = A.host;
  const int64_t n = H.n, ns = (n + 31) / 32;
  std::vector<int64_t> off(ns + 1, 0);
  for (int64_t sl = 0; sl < ns; ++sl) {
    int64_t w = 0;
    for (int64_t r = sl * 32; r < std::min(n, sl * 32 + 32); ++r) w = std::max(w, H.rp[r + 1] - H.rp[r]);
    off[sl + 1] = off[sl] + 32 * w;
  }
  std::vector<int32_t> ci(off[ns]);
  std::vector<double> v(off[ns], 0.0);
  parallel_for(ns, [&](int64_t s0, int64_t s1) {
    for (int64_t sl = s0; sl < s1; ++sl) {
      const int64_t w = (off[sl + 1] - off[sl]) / 32;
      for (int t = 0; t < 32; ++t) {
        const int64_t r = sl * 32 + t;
        const int64_t len = r < n ? H.rp[r + 1] - H.rp[r] : 0;
        for (int64_t j = 0; j < w; ++j) {
          const int64_t o = off[sl] + 32 * j + t;
          if (j < len) {
            ci[o] = (int32_t)H.ci[H.rp[r] + j];
            v[o] = H.v[H.rp[r] + j];
          } else {
            ci[o] = (int32_t)std::min<int64_t>(r, n - 1);
            v[o] = 0.0;
          }
        }
      }
    }
  }, 1 << 12);
  A.sell_off.upload(off.data(), ns + 1);
  A.sell_ci.upload(ci.data(), off[ns]);
  A.sell_v.upload(v.data(), off[ns]);
  RCHOL_CUDA(cudaDeviceSynchronize());
}

namespace {

// ---- PCG --------------------------------------------------------------------------
//
// Per right-hand side r the device keeps: bnorm2, rnorm2, rz, rz_prev, pr, pq,
// alpha, beta, active, iters.  Every reduction is deterministic: a fixed grid,
// a fixed per-thread assignment, fixed-shape trees.

constexpr int RED_BLOCKS = 512;
constexpr int RED_THREADS = 256;

struct PcgState {
  double *bnorm2, *rnorm2, *rz, *rz_prev, *pr, *pq, *alpha, *beta;
  int *active, *iters;
  int *any_active;
  double *partial;  // RED_BLOCKS * k * 2
  int k;
  const double *tol;  // in device memory so that a captured graph serves any call
  const int *maxit;
};

enum RedOp { RED_DOT = 0, RED_DOT2 = 1, RED_UPDATE = 2, RED_RESID = 3 };

// Generic per-RHS reduction over rows.  Thread mapping: rhs = t % k,
// row lane = t / k with a power-of-two number of row lanes per block.
template <int OP>
__global__ void __launch_bounds__(RED_THREADS) reduce_kernel(int64_t n, PcgState st, const double *a,
                                                             const double *b, double *c, double *d,
                                                             const double *e) {
  __shared__ double sh[2][RED_THREADS];
  const int k = st.k;
  if (OP != RED_RESID && !*st.any_active) return;
  int lanes = 1;
  while (lanes * 2 * k <= RED_THREADS) lanes *= 2;
  const int t = threadIdx.x;
  const int r = t % k, rl = t / k;
  const bool act_t = (k <= RED_THREADS) && (rl < lanes);
  int64_t per = (n + gridDim.x - 1) / gridDim.x;
  int64_t i0 = blockIdx.x * per, i1 = min(n, i0 + per);
  double s0 = 0.0, s1 = 0.0;
  if (act_t) {
    if (OP == RED_DOT) {  // s0 = a.b
      for (int64_t i = i0 + rl; i < i1; i += lanes) s0 += a[i * k + r] * b[i * k + r];
    } else if (OP == RED_DOT2) {  // s0 = a.b, s1 = a.e  (p.q and p.r)
      for (int64_t i = i0 + rl; i < i1; i += lanes) {
        double pv = a[i * k + r];
        s0 += pv * b[i * k + r];
        s1 += pv * e[i * k + r];
      }
    } else if (OP == RED_UPDATE) {  // x += alpha p ; r -= alpha q ; s0 = r.r
      double al = st.active[r] ? st.alpha[r] : 0.0;
      bool on = st.active[r];
      for (int64_t i = i0 + rl; i < i1; i += lanes) {
        int64_t o = i * k + r;
        double rv = d[o];
        if (on) {
          c[o] += al * a[o];
          rv += -al * b[o];
          d[o] = rv;
        }
        s0 += rv * rv;
      }
    } else {  // RED_RESID: s0 = (a - b).(a - b)  with a = A x, b = rhs
      for (int64_t i = i0 + rl; i < i1; i += lanes) {
        double q = a[i * k + r] + -1.0 * b[i * k + r];
        s0 += q * q;
      }
    }
  }
  sh[0][t] = s0;
  sh[1][t] = s1;
  __syncthreads();
  for (int h = lanes / 2; h > 0; h >>= 1) {
    if (act_t && rl < h) {
      sh[0][t] += sh[0][t + h * k];
      sh[1][t] += sh[1][t + h * k];
    }
    __syncthreads();
  }
  if (act_t && rl == 0) {
    st.partial[(int64_t)blockIdx.x * k + r] = sh[0][t];
    st.partial[(int64_t)(gridDim.x + blockIdx.x) * k + r] = sh[1][t];
  }
}

// Sum the RED_BLOCKS partials of every rhs (one block per rhs, fixed tree).
__device__ double block_total(const double *part, int k, int r, int which) {
  __shared__ double sh[RED_THREADS];
  double s = 0.0;
  for (int bb = threadIdx.x; bb < RED_BLOCKS; bb += RED_THREADS)
    s += part[(int64_t)(which * RED_BLOCKS + bb) * k + r];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int h = RED_THREADS / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  double tot = sh[0];
  __syncthreads();
  return tot;
}

enum FinOp { FIN_INIT = 0, FIN_BETA = 1, FIN_ALPHA = 2, FIN_CONV = 3, FIN_RESID = 4 };

__global__ void finalize_kernel(PcgState st, int op, int first, double *relres) {
  const int r = blockIdx.x;
  if (op != FIN_INIT && op != FIN_RESID && !*st.any_active) return;
  double t0 = block_total(st.partial, st.k, r, 0);
  double t1 = block_total(st.partial, st.k, r, 1);
  if (threadIdx.x != 0) return;
  if (op == FIN_INIT) {  // t0 = b.b (r = b)
    st.bnorm2[r] = t0;
    st.rnorm2[r] = t0;
    st.iters[r] = 0;
    int act = (sqrt(t0) > sqrt(t0) * *st.tol) && (*st.maxit > 0);
    st.active[r] = act;
    if (act) atomicOr(st.any_active, 1);
  } else if (op == FIN_BETA) {  // t0 = r.z
    if (st.active[r]) {
      st.beta[r] = st.iters[r] == 0 ? 0.0 : t0 / st.rz_prev[r];
      st.rz[r] = t0;
    }
  } else if (op == FIN_ALPHA) {  // t0 = p.q, t1 = p.r
    if (st.active[r]) {
      st.pq[r] = t0;
      st.pr[r] = t1;
      st.alpha[r] = t1 / t0;
    }
  } else if (op == FIN_CONV) {  // t0 = r.r after the update
    if (st.active[r]) {
      st.rnorm2[r] = t0;
      st.rz_prev[r] = st.rz[r];
      int it = st.iters[r] + 1;
      st.iters[r] = it;
      st.active[r] = (sqrt(t0) > sqrt(st.bnorm2[r]) * *st.tol) && (it < *st.maxit);
    }
  } else {  // FIN_RESID
    relres[r] = sqrt(t0) / sqrt(st.bnorm2[r]);
  }
}

__global__ void any_active_kernel(PcgState st) {
  int a = 0;
  for (int r = 0; r < st.k; ++r) a |= st.active[r];
  *st.any_active = a;
}

// p = beta p + z (p = z on the first iteration), only for active right-hand sides.
__global__ void pupdate_kernel(int64_t nk, PcgState st, double *p, const double *z) {
  if (!*st.any_active) return;
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nk) return;
  int r = (int)(i % st.k);
  if (!st.active[r]) return;
  if (st.iters[r] == 0) p[i] = z[i];
  else p[i] = st.beta[r] * p[i] + 1.0 * z[i];
}

__global__ void init_kernel(int64_t nk, const double *b, double *x, double *r) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= nk) return;
  x[i] = 0.0;
  r[i] = b[i];
}

}  // namespace

// ---- plan construction -----------------------------------------------------------

namespace {

__global__ void transpose_count_kernel(int64_t nnz, const int32_t *uci, unsigned long long *cnt) {
  int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (q < nnz) atomicAdd(&cnt[uci[q]], 1ull);
}

__global__ void transpose_scatter_kernel(int64_t n, const int64_t *urp, const int32_t *uci,
                                         const double *uv, const int64_t *lrp,
                                         unsigned long long *cur, int32_t *tci, double *tv) {
  int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= n) return;
  for (int64_t q = urp[row] + lane; q < urp[row + 1]; q += 32) {
    int32_t j = uci[q];
    unsigned long long slot = atomicAdd(&cur[j], 1ull);
    tci[lrp[j] + slot] = (int32_t)row;
    tv[lrp[j] + slot] = uv[q];
  }
}

// Sort each row of L by column (rank sort; columns within a row are unique).
__global__ void row_sort_kernel(int64_t n, const int64_t *lrp, const int32_t *tci, const double *tv,
                                int32_t *lci, double *lv) {
  int64_t row = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (row >= n) return;
  int64_t b = lrp[row], e = lrp[row + 1];
  for (int64_t q = b + lane; q < e; q += 32) {
    int32_t c = tci[q];
    int64_t rank = 0;
    for (int64_t f = b; f < e; ++f) rank += (tci[f] < c);
    lci[b + rank] = c;
    lv[b + rank] = tv[q];
  }
}


__global__ void to_f32_kernel(int64_t n, const double *a, float *b) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (float)a[i];
}

__global__ void i64_from_ull_kernel(int64_t n, const unsigned long long *a, int64_t *b) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = (int64_t)a[i];
}

}  // namespace

void finish_factor(rchol_factor_s &F, cudaStream_t s) {
  const int64_t n = F.n, nnz = F.nnz;
  const auto t0 = std::chrono::steady_clock::now();
  // L = transpose(U)
  DevBuf<unsigned long long> cnt(n);
  RCHOL_CUDA(cudaMemsetAsync(cnt.p, 0, cnt.bytes(), s));
  transpose_count_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, F.uci.p, cnt.p);
  note_launch();
  F.lrp.alloc(n + 1);
  i64_from_ull_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(n, cnt.p, F.lrp.p);
  note_launch();
  RCHOL_CUDA(cudaGetLastError());
  exclusive_scan_i64(F.lrp.p, n, s);
  RCHOL_CUDA(cudaMemsetAsync(cnt.p, 0, cnt.bytes(), s));
  {
    DevBuf<int32_t> tci(nnz);
    DevBuf<double> tv(nnz);
    transpose_scatter_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(
        n, F.urp.p, F.uci.p, F.uv.p, F.lrp.p, cnt.p, tci.p, tv.p);
    note_launch();
    F.lci.alloc(nnz);
    F.lv.alloc(nnz);
    row_sort_kernel<<<(unsigned)((n * 32 + 255) / 256), 256, 0, s>>>(n, F.lrp.p, tci.p, tv.p, F.lci.p,
                                                                      F.lv.p);
    note_launch();
    RCHOL_CUDA(cudaGetLastError());
    RCHOL_CUDA(cudaStreamSynchronize(s));
  }
  if (F.precision == RCHOL_PREC_FP32) {
    F.uv32.alloc(nnz);
    F.lv32.alloc(nnz);
    to_f32_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, F.uv.p, F.uv32.p);
    note_launch();
    to_f32_kernel<<<(unsigned)((nnz + 255) / 256), 256, 0, s>>>(nnz, F.lv.p, F.lv32.p);
    note_launch();
    RCHOL_CUDA(cudaGetLastError());
  }
  RCHOL_CUDA(cudaStreamSynchronize(s));
  const auto t1 = std::chrono::steady_clock::now();
  build_plan(F, s);
  RCHOL_CUDA(cudaStreamSynchronize(s));
  F.t_assemble = std::chrono::duration<double>(t1 - t0).count();
  F.t_plan = std::chrono::duration<double>(std::chrono::steady_clock::now() - t1).count();
}

void build_plan(rchol_factor_s &F, cudaStream_t s) {
  auto P = new SolvePlan();
  try {
    build_streams(F, *P, s);
  } catch (...) {
    delete P;
    throw;
  }
  destroy_plan(F.plan);
  F.plan = P;
}

// Grows the plan's temporaries.  Growing frees buffers that captured PCG
// graphs point to, so every cached graph of this factor is dropped with them
// (a replay would otherwise read and write freed memory).  Callers hold P.lock.
static void ensure_scratch(SolvePlan &P, bool fp32, int64_t count) {
  bool grew = false;
  if (fp32) {
    if (P.ytmp32.n < (size_t)count) P.ytmp32.alloc(count), grew = true;
  } else {
    if (P.ytmp.n < (size_t)count) P.ytmp.alloc(count), grew = true;
  }
  if (grew) {
    P.pcg.clear();
    P.seg.clear();
  }
}

// The preconditioner with the plan's buffers already sized (inside PCG).
static void precond_ready(const rchol_factor_s &F, const double *r, double *z, int k, cudaStream_t s);

void trsv(const rchol_factor_s &F, bool upper, const double *in, double *out, int k, cudaStream_t s) {
  SolvePlan &P = *F.plan;
  std::lock_guard<std::mutex> guard(P.lock);
  ensure_scratch(P, F.precision == RCHOL_PREC_FP32, F.n * k);
  if (k == 1) {
    stream_trsv(F, P, upper, in, nullptr, out, nullptr, s);
    return;
  }
  build_streams_k(F, P, s);
  stream_trsv_k(F, P, upper, in, nullptr, out, nullptr, k, s);
}

void precond(const rchol_factor_s &F, const double *r, double *z, int k, cudaStream_t s) {
  SolvePlan &P = *F.plan;
  std::lock_guard<std::mutex> guard(P.lock);
  ensure_scratch(P, F.precision == RCHOL_PREC_FP32, F.n * k);
  if (k > 1) build_streams_k(F, P, s);
  precond_ready(F, r, z, k, s);
}

static void precond_ready(const rchol_factor_s &F, const double *r, double *z, int k, cudaStream_t s) {
  SolvePlan &P = *F.plan;
  const bool fp32 = F.precision == RCHOL_PREC_FP32;
  if (k == 1) {
    if (fp32) {
      stream_trsv(F, P, false, r, nullptr, nullptr, P.ytmp32.p, s);
      stream_trsv(F, P, true, nullptr, P.ytmp32.p, z, nullptr, s);
    } else {
      stream_trsv(F, P, false, r, nullptr, P.ytmp.p, nullptr, s);
      stream_trsv(F, P, true, P.ytmp.p, nullptr, z, nullptr, s);
    }
    return;
  }
  if (fp32) {
    stream_trsv_k(F, P, false, r, nullptr, nullptr, P.ytmp32.p, k, s);
    stream_trsv_k(F, P, true, nullptr, P.ytmp32.p, z, nullptr, k, s);
  } else {
    stream_trsv_k(F, P, false, r, nullptr, P.ytmp.p, nullptr, k, s);
    stream_trsv_k(F, P, true, P.ytmp.p, nullptr, z, nullptr, k, s);
  }
}

void spmv_public(const rchol_matrix_s &A, const double *x, double *y, int k, cudaStream_t s) {
  spmv(A, x, y, k, s);
}

namespace {
// dL/dw_e = -(lambda_i - lambda_j)(x_i - x_j): the derivative of -lambda^T A(w) x
// with respect to one edge weight.
__global__ void edge_grad_kernel(int64_t m, const int64_t *__restrict__ ei, const int64_t *__restrict__ ej,
                                 const double *__restrict__ lam, const double *__restrict__ x,
                                 double *__restrict__ g) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= m) return;
  const int64_t i = ei[e], j = ej[e];
  g[e] = -(lam[i] - lam[j]) * (x[i] - x[j]);
}
}  // namespace

void edge_grad(int64_t m, const int64_t *ei, const int64_t *ej, const double *lam, const double *x, double *g,
               cudaStream_t s) {
  if (m <= 0) return;
  edge_grad_kernel<<<(unsigned)((m + 255) / 256), 256, 0, s>>>(m, ei, ej, lam, x, g);
  note_launch();
  RCHOL_CUDA(cudaGetLastError());
}

// Longest dependency chain (levels of a level schedule) of the forward or
// backward solve, computed on first request from the CSR of G or G^T.
int64_t plan_levels(const rchol_factor_s &F, bool upper) {
  SolvePlan &P = *F.plan;
  std::lock_guard<std::mutex> guard(P.lock);
  int64_t &dag = upper ? P.dag_bwd : P.dag_fwd;
  if (dag >= 0) return dag;
  const int64_t n = F.n, nnz = F.nnz;
  std::vector<int64_t> rp(n + 1);
  std::vector<int32_t> ci(nnz);
  (upper ? F.urp : F.lrp).download(rp.data(), n + 1, 0);
  (upper ? F.uci : F.lci).download(ci.data(), nnz, 0);
  RCHOL_CUDA(cudaStreamSynchronize(0));
  std::vector<int32_t> lv(n, 0);
  int32_t mx = 0;
  if (!upper) {  // rows of G: diagonal last
    for (int64_t i = 0; i < n; ++i) {
      int32_t l = 0;
      for (int64_t q = rp[i]; q < rp[i + 1] - 1; ++q) l = std::max(l, lv[ci[q]] + 1);
      lv[i] = l;
      mx = std::max(mx, l);
    }
  } else {  // rows of G^T: diagonal first
    for (int64_t i = n - 1; i >= 0; --i) {
      int32_t l = 0;
      for (int64_t q = rp[i] + 1; q < rp[i + 1]; ++q) l = std::max(l, lv[ci[q]] + 1);
      lv[i] = l;
      mx = std::max(mx, l);
    }
  }
  dag = n ? (int64_t)mx + 1 : 0;
  return dag;
}

// PCG for k right-hand sides (device pointers), c++/util/pcg.cpp:57-127.
//
// One iteration (preconditioner, r.z, p update, SpMV with p.q and p.r, x/r
// update with ||r||^2, stopping test) is captured once per (matrix, factor, k)
// into a CUDA graph and replayed; every kernel returns at once when no
// right-hand side is active any more, so the host checks convergence only
// every few iterations.  The graph runs on the workspace's own stream, joined
// to the caller's stream with events.
static PcgWork &pcg_workspace(const rchol_matrix_s &A, const rchol_factor_s &F, int k) {
  SolvePlan &P = *F.plan;
  for (auto &w : P.pcg)
    if (w->key_uid == A.uid && w->n == A.n && w->nnz == A.nnz && w->k == k)
      return *w;
  if (P.pcg.size() >= 4) P.pcg.erase(P.pcg.begin());
  auto w = std::make_unique<PcgWork>();
  w->key_uid = A.uid;
  w->n = A.n;
  w->nnz = A.nnz;
  w->k = k;
  const int64_t nk = A.n * k;
  w->r.alloc(nk);
  w->z.alloc(nk);
  w->p.alloc(nk);
  w->q.alloc(nk);
  w->x.alloc(nk);
  w->sc.alloc(9 * (size_t)k + 2 * (size_t)RED_BLOCKS * k + 1);
  w->ic.alloc(2 * (size_t)k + 2);
  RCHOL_CUDA(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
  RCHOL_CUDA(cudaEventCreateWithFlags(&w->ev_in, cudaEventDisableTiming));
  RCHOL_CUDA(cudaEventCreateWithFlags(&w->ev_out, cudaEventDisableTiming));
  P.pcg.push_back(std::move(w));
  return *P.pcg.back();
}

static PcgState pcg_state(PcgWork &w) {
  const int k = w.k;
  PcgState st;
  double *sc = w.sc.p;
  st.bnorm2 = sc;
  st.rnorm2 = sc + k;
  st.rz = sc + 2 * k;
  st.rz_prev = sc + 3 * k;
  st.pr = sc + 4 * k;
  st.pq = sc + 5 * k;
  st.alpha = sc + 6 * k;
  st.beta = sc + 7 * k;
  st.partial = sc + 8 * k;
  // [8k, 8k + 2*RB*k) partial sums, then k relres slots, then tol
  st.tol = sc + 9 * k + 2 * (size_t)RED_BLOCKS * k;
  st.active = w.ic.p;
  st.iters = w.ic.p + k;
  st.any_active = w.ic.p + 2 * k;
  st.maxit = w.ic.p + 2 * k + 1;
  st.k = k;
  return st;
}

static void pcg_iteration(const rchol_matrix_s &A, const rchol_factor_s &F, PcgWork &w, const PcgState &st,
                          cudaStream_t s) {
  const int k = w.k;
  const int64_t n = A.n, nk = n * k;
  const unsigned eb = (unsigned)((nk + 255) / 256);
  precond_ready(F, w.r.p, w.z.p, k, s);
  reduce_kernel<RED_DOT><<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, st, w.r.p, w.z.p, nullptr, nullptr, nullptr);
  finalize_kernel<<<k, RED_THREADS, 0, s>>>(st, FIN_BETA, 0, nullptr);
  pupdate_kernel<<<eb, 256, 0, s>>>(nk, st, w.p.p, w.z.p);
  spmv(A, w.p.p, w.q.p, k, s);
  reduce_kernel<RED_DOT2><<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, st, w.p.p, w.q.p, nullptr, nullptr, w.r.p);
  finalize_kernel<<<k, RED_THREADS, 0, s>>>(st, FIN_ALPHA, 0, nullptr);
  reduce_kernel<RED_UPDATE><<<RED_BLOCKS, RED_THREADS, 0, s>>>(n, st, w.p.p, w.q.p, w.x.p, w.r.p, nullptr);
  finalize_kernel<<<k, RED_THREADS, 0, s>>>(st, FIN_CONV, 0, nullptr);
  any_active_kernel<<<1, 1, 0, s>>>(st);
  RCHOL_CUDA(cudaGetLastError());
}

// b_host / x_host: the host-buffer entry point (b copied in and x copied out
// on the workspace stream, through device staging kept with the workspace).
static void pcg_impl(const rchol_matrix_s &A, const rchol_factor_s &F, const double *b, double *x,
                     const double *b_host, double *x_host, int k, double tol, int maxit, double *relres,
                     int *itr, cudaStream_t s) {
  SolvePlan &P = *F.plan;
  std::lock_guard<std::mutex> guard(P.lock);
  const int64_t n = A.n, nk = n * k;
  const bool fp32 = F.precision == RCHOL_PREC_FP32;
  ensure_scratch(P, fp32, nk);
  if (k > 1) build_streams_k(F, P, s);
  if (fp32 ? P.acc32.n < (size_t)n : P.acc64.n < (size_t)n) {
    if (fp32) P.acc32.alloc(n);
    else P.acc64.alloc(n);
  }
  PcgWork &w = pcg_workspace(A, F, k);
  PcgState st = pcg_state(w);
  cudaStream_t ws = w.stream;
  RCHOL_CUDA(cudaEventRecord(w.ev_in, s));
  RCHOL_CUDA(cudaStreamWaitEvent(ws, w.ev_in, 0));
  if (b_host) {
    if (w.hb.n < (size_t)nk) w.hb.alloc(nk);
    if (w.hx.n < (size_t)nk) w.hx.alloc(nk);
    RCHOL_CUDA(cudaMemcpyAsync(w.hb.p, b_host, nk * sizeof(double), cudaMemcpyHostToDevice, ws));
    b = w.hb.p;
    x = w.hx.p;
  }
  if (!w.exec) {
    cudaGraph_t g = nullptr;
    RCHOL_CUDA(cudaStreamBeginCapture(ws, cudaStreamCaptureModeThreadLocal));
    try {
      pcg_iteration(A, F, w, st, ws);
    } catch (...) {
      cudaStreamEndCapture(ws, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    RCHOL_CUDA(cudaStreamEndCapture(ws, &g));
    size_t nodes = 0;
    RCHOL_CUDA(cudaGraphGetNodes(g, nullptr, &nodes));
    w.graph_kernels = (int64_t)nodes;
    cudaError_t e = cudaGraphInstantiate(&w.exec, g, 0);
    cudaGraphDestroy(g);
    RCHOL_CUDA(e);
  }
  // setup: tolerances, x = 0, r = b, ||b||^2 and the initial stopping test
  double htol = tol;
  int hmax = maxit;
  RCHOL_CUDA(cudaMemsetAsync(w.sc.p, 0, w.sc.bytes(), ws));
  RCHOL_CUDA(cudaMemsetAsync(w.ic.p, 0, w.ic.bytes(), ws));
  RCHOL_CUDA(cudaMemcpyAsync(const_cast<double *>(st.tol), &htol, sizeof(double), cudaMemcpyHostToDevice, ws));
  RCHOL_CUDA(cudaMemcpyAsync(const_cast<int *>(st.maxit), &hmax, sizeof(int), cudaMemcpyHostToDevice, ws));
  const unsigned eb = (unsigned)((nk + 255) / 256);
  init_kernel<<<eb, 256, 0, ws>>>(nk, b, w.x.p, w.r.p);
  RCHOL_CUDA(cudaMemsetAsync(w.q.p, 0, w.q.bytes(), ws));
  reduce_kernel<RED_RESID><<<RED_BLOCKS, RED_THREADS, 0, ws>>>(n, st, b, w.q.p, nullptr, nullptr, nullptr);
  finalize_kernel<<<k, RED_THREADS, 0, ws>>>(st, FIN_INIT, 0, nullptr);
  note_launch(3);
  RCHOL_CUDA(cudaGetLastError());
  int h_any = 1;
  for (int it = 0; it < maxit;) {
    const int batch = it == 0 ? 8 : 4;
    for (int j = 0; j < batch && it < maxit; ++j, ++it) {
      RCHOL_CUDA(cudaGraphLaunch(w.exec, ws));
      note_launch(w.graph_kernels);
    }
    RCHOL_CUDA(cudaMemcpyAsync(&h_any, st.any_active, sizeof(int), cudaMemcpyDeviceToHost, ws));
    RCHOL_CUDA(cudaStreamSynchronize(ws));
    if (!h_any) break;
  }
  // x out, relres = ||A x - b|| / ||b||
  double *d_relres = w.sc.p + 8 * (size_t)k + 2 * (size_t)RED_BLOCKS * k;
  spmv(A, w.x.p, w.q.p, k, ws);
  reduce_kernel<RED_RESID><<<RED_BLOCKS, RED_THREADS, 0, ws>>>(n, st, w.q.p, b, nullptr, nullptr, nullptr);
  finalize_kernel<<<k, RED_THREADS, 0, ws>>>(st, FIN_RESID, 0, d_relres);
  note_launch(3);
  RCHOL_CUDA(cudaGetLastError());
  if (x_host) RCHOL_CUDA(cudaMemcpyAsync(x_host, w.x.p, nk * sizeof(double), cudaMemcpyDeviceToHost, ws));
  else RCHOL_CUDA(cudaMemcpyAsync(x, w.x.p, nk * sizeof(double), cudaMemcpyDeviceToDevice, ws));
  RCHOL_CUDA(cudaMemcpyAsync(relres, d_relres, k * sizeof(double), cudaMemcpyDeviceToHost, ws));
  RCHOL_CUDA(cudaMemcpyAsync(itr, st.iters, k * sizeof(int), cudaMemcpyDeviceToHost, ws));
  RCHOL_CUDA(cudaEventRecord(w.ev_out, ws));
  RCHOL_CUDA(cudaStreamWaitEvent(s, w.ev_out, 0));
  RCHOL_CUDA(cudaStreamSynchronize(ws));
}

void pcg_device(const rchol_matrix_s &A, const rchol_factor_s &F, const double *b, double *x, int k, double tol,
                int maxit, double *relres, int *itr, cudaStream_t s) {
  pcg_impl(A, F, b, x, nullptr, nullptr, k, tol, maxit, relres, itr, s);
}

void pcg_host(const rchol_matrix_s &A, const rchol_factor_s &F, const double *b, double *x, int k, double tol,
              int maxit, double *relres, int *itr) {
  pcg_impl(A, F, nullptr, nullptr, b, x, k, tol, maxit, relres, itr, 0);
}

// ---- batched PCG over independent systems ---------------------------------------------
//
// The systems are the diagonal blocks of one matrix (rows seg[s] .. seg[s+1])
// with a block-diagonal factor, so one SpMV and one preconditioner apply serve
// them all; the scalars of c++/util/pcg.cpp:57-127 are kept per system, one
// thread block per system computes them (fixed reduction trees, so results
// are deterministic), and a system stops updating once it has converged.

namespace {

constexpr int SEG_THREADS = 256;

struct SegState {
  const int64_t *seg;
  int nseg;
  double *bnorm2, *rz, *rz_prev, *relres;
  int *active, *iters, *any_active;
  const double *tol;
  const int *maxit;
};

// Block-wide sum in a fixed tree; every thread gets the total.
__device__ double seg_sum(double v, double *sh) {
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int h = SEG_THREADS / 2; h > 0; h >>= 1) {
    if (threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  const double t = sh[0];
  __syncthreads();
  return t;
}

// x = 0, r = b, ||b||^2 and the first stopping test (pcg.cpp:60-70).
__global__ void __launch_bounds__(SEG_THREADS) seg_init_kernel(SegState st, const double *b, double *x,
                                                               double *r) {
  __shared__ double sh[SEG_THREADS];
  const int s = blockIdx.x;
  const int64_t i0 = st.seg[s], i1 = st.seg[s + 1];
  double acc = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += SEG_THREADS) {
    const double bv = b[i];
    x[i] = 0.0;
    r[i] = bv;
    acc += bv * bv;
  }
  const double t = seg_sum(acc, sh);
  if (threadIdx.x == 0) {
    st.bnorm2[s] = t;
    st.iters[s] = 0;
    const int act = (sqrt(t) > sqrt(t) * *st.tol) && (*st.maxit > 0);
    st.active[s] = act;
    if (act) atomicOr(st.any_active, 1);
  }
}

// rz = r.z, beta = rz / rz_prev, p = z (first iteration) or beta p + z.
__global__ void __launch_bounds__(SEG_THREADS) seg_beta_kernel(SegState st, const double *r, const double *z,
                                                               double *p) {
  __shared__ double sh[SEG_THREADS];
  if (!*st.any_active) return;
  const int s = blockIdx.x;
  if (!st.active[s]) return;
  const int64_t i0 = st.seg[s], i1 = st.seg[s + 1];
  double acc = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += SEG_THREADS) acc += r[i] * z[i];
  const double rz = seg_sum(acc, sh);
  const int it = st.iters[s];
  const double beta = it == 0 ? 0.0 : rz / st.rz_prev[s];
  for (int64_t i = i0 + threadIdx.x; i < i1; i += SEG_THREADS) p[i] = it == 0 ? z[i] : beta * p[i] + 1.0 * z[i];
  if (threadIdx.x == 0) st.rz[s] = rz;
}

// alpha = p.r / p.q, x += alpha p, r -= alpha q, then the stopping test.
__global__ void __launch_bounds__(SEG_THREADS) seg_alpha_kernel(SegState st, const double *p, const double *q,
                                                                double *x, double *r) {
  __shared__ double sh[SEG_THREADS];
  if (!*st.any_active) return;
  const int s = blockIdx.x;
  if (!st.active[s]) return;
  const int64_t i0 = st.seg[s], i1 = st.seg[s + 1];
  double a0 = 0.0, a1 = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += SEG_THREADS) {
    const double pv = p[i];
    a0 += pv * q[i];
    a1 += pv * r[i];
  }
  const double pq = seg_sum(a0, sh);
  const double pr = seg_sum(a1, sh);
  const double alpha = pr / pq;
  double rr = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += SEG_THREADS) {
    x[i] += alpha * p[i];
    const double rv = r[i] + -alpha * q[i];
    r[i] = rv;
    rr += rv * rv;
  }
  const double t = seg_sum(rr, sh);
  if (threadIdx.x == 0) {
    const int it = st.iters[s] + 1;
    st.iters[s] = it;
    st.rz_prev[s] = st.rz[s];
    st.active[s] = (sqrt(t) > sqrt(st.bnorm2[s]) * *st.tol) && (it < *st.maxit);
  }
}

__global__ void seg_any_kernel(SegState st) {
  __shared__ int any;
  if (threadIdx.x == 0) any = 0;
  __syncthreads();
  int a = 0;
  for (int s = threadIdx.x; s < st.nseg; s += blockDim.x) a |= st.active[s];
  if (a) atomicOr(&any, 1);
  __syncthreads();
  if (threadIdx.x == 0) *st.any_active = any;
}

// relres = ||A x - b|| / ||b|| per system (q = A x).
__global__ void __launch_bounds__(SEG_THREADS) seg_resid_kernel(SegState st, const double *q, const double *b) {
  __shared__ double sh[SEG_THREADS];
  const int s = blockIdx.x;
  const int64_t i0 = st.seg[s], i1 = st.seg[s + 1];
  double acc = 0.0;
  for (int64_t i = i0 + threadIdx.x; i < i1; i += SEG_THREADS) {
    const double d = q[i] + -1.0 * b[i];
    acc += d * d;
  }
  const double t = seg_sum(acc, sh);
  if (threadIdx.x == 0) st.relres[s] = sqrt(t) / sqrt(st.bnorm2[s]);
}

}  // namespace

static SegWork &seg_workspace(const rchol_matrix_s &A, const rchol_factor_s &F, int64_t nseg,
                              const int64_t *seg) {
  SolvePlan &P = *F.plan;
  for (auto &w : P.seg)
    if (w->key_uid == A.uid && (int64_t)w->seg_host.size() == nseg + 1 &&
        std::equal(w->seg_host.begin(), w->seg_host.end(), seg))
      return *w;
  if (P.seg.size() >= 4) P.seg.erase(P.seg.begin());
  auto w = std::make_unique<SegWork>();
  w->key_uid = A.uid;
  w->seg_host.assign(seg, seg + nseg + 1);
  w->n = A.n;
  w->seg.upload(seg, nseg + 1, 0);
  w->r.alloc(A.n);
  w->z.alloc(A.n);
  w->p.alloc(A.n);
  w->q.alloc(A.n);
  w->x.alloc(A.n);
  w->sc.alloc(4 * (size_t)nseg + 1);
  w->ic.alloc(2 * (size_t)nseg + 2);
  RCHOL_CUDA(cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking));
  RCHOL_CUDA(cudaEventCreateWithFlags(&w->ev_in, cudaEventDisableTiming));
  RCHOL_CUDA(cudaEventCreateWithFlags(&w->ev_out, cudaEventDisableTiming));
  RCHOL_CUDA(cudaStreamSynchronize(0));
  P.seg.push_back(std::move(w));
  return *P.seg.back();
}

static SegState seg_state(SegWork &w) {
  const int S = (int)(w.seg_host.size() - 1);
  SegState st;
  st.seg = w.seg.p;
  st.nseg = S;
  st.bnorm2 = w.sc.p;
  st.rz = w.sc.p + S;
  st.rz_prev = w.sc.p + 2 * (size_t)S;
  st.relres = w.sc.p + 3 * (size_t)S;
  st.tol = w.sc.p + 4 * (size_t)S;
  st.active = w.ic.p;
  st.iters = w.ic.p + S;
  st.any_active = w.ic.p + 2 * (size_t)S;
  st.maxit = w.ic.p + 2 * (size_t)S + 1;
  return st;
}

static void pcg_batch_impl(const rchol_matrix_s &A, const rchol_factor_s &F, int64_t nseg, const int64_t *seg,
                           const double *b, double *x, const double *b_host, double *x_host, double tol,
                           int maxit, double *relres, int *itr, cudaStream_t s) {
  SolvePlan &P = *F.plan;
  std::lock_guard<std::mutex> guard(P.lock);
  const int64_t n = A.n;
  const bool fp32 = F.precision == RCHOL_PREC_FP32;
  ensure_scratch(P, fp32, n);
  if (fp32 ? P.acc32.n < (size_t)n : P.acc64.n < (size_t)n) {
    if (fp32) P.acc32.alloc(n);
    else P.acc64.alloc(n);
  }
  SegWork &w = seg_workspace(A, F, nseg, seg);
  SegState st = seg_state(w);
  const unsigned S = (unsigned)nseg;
  cudaStream_t ws = w.stream;
  RCHOL_CUDA(cudaEventRecord(w.ev_in, s));
  RCHOL_CUDA(cudaStreamWaitEvent(ws, w.ev_in, 0));
  if (b_host) {
    if (w.hb.n < (size_t)n) w.hb.alloc(n);
    if (w.hx.n < (size_t)n) w.hx.alloc(n);
    RCHOL_CUDA(cudaMemcpyAsync(w.hb.p, b_host, n * sizeof(double), cudaMemcpyHostToDevice, ws));
    b = w.hb.p;
    x = w.hx.p;
  }
  if (!w.exec) {
    cudaGraph_t g = nullptr;
    RCHOL_CUDA(cudaStreamBeginCapture(ws, cudaStreamCaptureModeThreadLocal));
    try {
      precond_ready(F, w.r.p, w.z.p, 1, ws);
      seg_beta_kernel<<<S, SEG_THREADS, 0, ws>>>(st, w.r.p, w.z.p, w.p.p);
      spmv(A, w.p.p, w.q.p, 1, ws);
      seg_alpha_kernel<<<S, SEG_THREADS, 0, ws>>>(st, w.p.p, w.q.p, w.x.p, w.r.p);
      seg_any_kernel<<<1, 256, 0, ws>>>(st);
      RCHOL_CUDA(cudaGetLastError());
    } catch (...) {
      cudaStreamEndCapture(ws, &g);
      if (g) cudaGraphDestroy(g);
      throw;
    }
    RCHOL_CUDA(cudaStreamEndCapture(ws, &g));
    size_t nodes = 0;
    RCHOL_CUDA(cudaGraphGetNodes(g, nullptr, &nodes));
    w.graph_kernels = (int64_t)nodes;
    cudaError_t e = cudaGraphInstantiate(&w.exec, g, 0);
    cudaGraphDestroy(g);
    RCHOL_CUDA(e);
  }
  double htol = tol;
  int hmax = maxit;
  RCHOL_CUDA(cudaMemsetAsync(w.sc.p, 0, w.sc.bytes(), ws));
  RCHOL_CUDA(cudaMemsetAsync(w.ic.p, 0, w.ic.bytes(), ws));
  RCHOL_CUDA(cudaMemcpyAsync(const_cast<double *>(st.tol), &htol, sizeof(double), cudaMemcpyHostToDevice, ws));
  RCHOL_CUDA(cudaMemcpyAsync(const_cast<int *>(st.maxit), &hmax, sizeof(int), cudaMemcpyHostToDevice, ws));
  seg_init_kernel<<<S, SEG_THREADS, 0, ws>>>(st, b, w.x.p, w.r.p);
  note_launch(1);
  RCHOL_CUDA(cudaGetLastError());
  int h_any = 1;
  for (int it = 0; it < maxit;) {
    const int batch = it == 0 ? 8 : 4;
    for (int j = 0; j < batch && it < maxit; ++j, ++it) {
      RCHOL_CUDA(cudaGraphLaunch(w.exec, ws));
      note_launch(w.graph_kernels);
    }
    RCHOL_CUDA(cudaMemcpyAsync(&h_any, st.any_active, sizeof(int), cudaMemcpyDeviceToHost, ws));
    RCHOL_CUDA(cudaStreamSynchronize(ws));
    if (!h_any) break;
  }
  spmv(A, w.x.p, w.q.p, 1, ws);
  seg_resid_kernel<<<S, SEG_THREADS, 0, ws>>>(st, w.q.p, b);
  note_launch(2);
  RCHOL_CUDA(cudaGetLastError());
  if (x_host) RCHOL_CUDA(cudaMemcpyAsync(x_host, w.x.p, n * sizeof(double), cudaMemcpyDeviceToHost, ws));
  else RCHOL_CUDA(cudaMemcpyAsync(x, w.x.p, n * sizeof(double), cudaMemcpyDeviceToDevice, ws));
  RCHOL_CUDA(cudaMemcpyAsync(relres, st.relres, nseg * sizeof(double), cudaMemcpyDeviceToHost, ws));
  RCHOL_CUDA(cudaMemcpyAsync(itr, st.iters, nseg * sizeof(int), cudaMemcpyDeviceToHost, ws));
  RCHOL_CUDA(cudaEventRecord(w.ev_out, ws));
  RCHOL_CUDA(cudaStreamWaitEvent(s, w.ev_out, 0));
  RCHOL_CUDA(cudaStreamSynchronize(ws));
}

void pcg_batch_device(const rchol_matrix_s &A, const rchol_factor_s &F, int64_t nseg, const int64_t *seg,
                      const double *b, double *x, double tol, int maxit, double *relres, int *itr,
                      cudaStream_t s) {
  pcg_batch_impl(A, F, nseg, seg, b, x, nullptr, nullptr, tol, maxit, relres, itr, s);
}

void pcg_batch_host(const rchol_matrix_s &A, const rchol_factor_s &F, int64_t nseg, const int64_t *seg,
                    const double *b, double *x, double tol, int maxit, double *relres, int *itr) {
  pcg_batch_impl(A, F, nseg, seg, nullptr, nullptr, b, x, tol, maxit, relres, itr, 0);
}

}  // namespace rchol
