// Shared definitions of the rchol_gb300 library: status handling, device
// buffers and the in-memory form of the three handles of include/rchol_gpu.h.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <stdexcept>
#include <string>
#include <vector>

#include "rchol_gpu.h"

namespace rchol {

// Error carrying an RCHOL_ERR_* status; the C ABI converts it to a return code.
struct Error : std::runtime_error {
  int status;
  Error(int s, const std::string &m) : std::runtime_error(m), status(s) {}
};

void set_last_error(const std::string &msg);
// Counts kernel launches made by the solve path (rchol_gpu_launch_count).
void note_launch(int64_t count = 1);

#define RCHOL_CUDA(call)                                                                  \
  do {                                                                                    \
    cudaError_t e_ = (call);                                                              \
    if (e_ != cudaSuccess)                                                                \
      throw ::rchol::Error(e_ == cudaErrorMemoryAllocation ? RCHOL_ERR_NOMEM : RCHOL_ERR_CUDA, \
                           std::string(#call) + ": " + cudaGetErrorString(e_));          \
  } while (0)

#define RCHOL_CHECK_ARG(cond, msg)                              \
  do {                                                          \
    if (!(cond)) throw ::rchol::Error(RCHOL_ERR_INVALID, (msg)); \
  } while (0)

// Owning device allocation.
template <typename T>
struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  explicit DevBuf(size_t count) { alloc(count); }
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  DevBuf(DevBuf &&o) noexcept : p(o.p), n(o.n) {
    o.p = nullptr;
    o.n = 0;
  }
  DevBuf &operator=(DevBuf &&o) noexcept {
    if (this != &o) {
      release();
      p = o.p;
      n = o.n;
      o.p = nullptr;
      o.n = 0;
    }
    return *this;
  }
  ~DevBuf() { release(); }
  void alloc(size_t count) {
    release();
    n = count;
    if (count) RCHOL_CUDA(cudaMalloc(&p, count * sizeof(T)));
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  size_t bytes() const { return n * sizeof(T); }
  void upload(const T *h, size_t count, cudaStream_t s = 0) {
    if (count > n) alloc(count);
    if (count) RCHOL_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
  }
  void download(T *h, size_t count, cudaStream_t s = 0) const {
    if (count) RCHOL_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
  }
};

// Host CSR with 64-bit row pointers and 64-bit column indices.
struct HostCsr {
  int64_t n = 0;
  std::vector<int64_t> rp, ci;
  std::vector<double> v;
  int64_t nnz() const { return rp.empty() ? 0 : rp.back(); }
};

// One node of the nested-dissection tree: a contiguous range of the ordered
// vertices.  Leaves are the subdomains, the others separators.
struct TreeNode {
  int64_t begin, end;  // [begin, end) in the new ordering (ground included in the root)
  int depth;           // 1 = root
  bool leaf;
};

}  // namespace rchol

// ---- handle bodies --------------------------------------------------------

struct rchol_tree_s {
  int64_t n = 0;
  int threads = 1;
  std::vector<int64_t> perm;  // new -> old
  std::vector<int64_t> part;  // result_idx (2*threads entries)
  std::vector<rchol::TreeNode> nodes;
  int depth = 1;  // number of tree levels
};

struct rchol_matrix_s {
  uint64_t uid = 0;  // unique per created matrix (keys cached solve workspaces)
  int64_t n = 0;
  int64_t nnz = 0;
  bool permuted = false;
  std::vector<int64_t> perm;    // empty when not permuted
  std::vector<int64_t> srcpos;  // stored entry q = caller's entry srcpos[q] (permuted only)
  rchol::HostCsr host;          // the stored (possibly permuted) matrix
  rchol::DevBuf<int64_t> rp;
  rchol::DevBuf<int32_t> ci;
  rchol::DevBuf<double> v;
  // Sliced ELL copy for single right-hand-side SpMV: 32-row slices, entry j
  // of row 32s+t at sell_off[s] + 32j + t (padding: column = row, value 0).
  rchol::DevBuf<int64_t> sell_off;
  rchol::DevBuf<int32_t> sell_ci;
  rchol::DevBuf<double> sell_v;
};

namespace rchol {
void build_sell(rchol_matrix_s &A);  // from A.host (solve.cu)
}

namespace rchol {
struct SolvePlan;  // triangular-solve schedule, defined in solve.cu
void destroy_plan(SolvePlan *);
}  // namespace rchol

struct rchol_factor_s {
  int64_t n = 0;
  int64_t nnz = 0;
  int precision = RCHOL_PREC_FP64;
  // U = CSR of G^T (row i = column i of G, diagonal first), as the reference returns G.
  rchol::DevBuf<int64_t> urp;
  rchol::DevBuf<int32_t> uci;
  rchol::DevBuf<double> uv;
  // L = CSR of G (row i = row i of G, diagonal last).
  rchol::DevBuf<int64_t> lrp;
  rchol::DevBuf<int32_t> lci;
  rchol::DevBuf<double> lv;
  // FP32 copies of the values when precision == FP32.
  rchol::DevBuf<float> uv32, lv32;
  rchol::DevBuf<double> pivots;  // d (length n), when produced by the GPU factorization
  std::vector<rchol::TreeNode> nodes;
  rchol::SolvePlan *plan = nullptr;
  // Wall time of the set-up phases (seconds): the elimination kernels, the
  // assembly of G (transpose, row sort, FP32 copies) and the solve plan.
  double t_eliminate = 0.0, t_assemble = 0.0, t_plan = 0.0;
  ~rchol_factor_s() { rchol::destroy_plan(plan); }
};
