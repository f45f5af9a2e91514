// Small device utilities: exclusive scans used by CSR assembly.

#include "common.hpp"

namespace rchol {

namespace {

constexpr int SCAN_THREADS = 1024;

__global__ void block_sums_kernel(const int64_t *in, int64_t n, int64_t per_block, int64_t *sums) {
  __shared__ int64_t red[SCAN_THREADS / 32];
  int64_t b0 = blockIdx.x * per_block, b1 = min(n, b0 + per_block);
  int64_t s = 0;
  for (int64_t i = b0 + threadIdx.x; i < b1; i += blockDim.x) s += in[i];
  for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    s = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0;
    for (int o = 16; o; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (threadIdx.x == 0) sums[blockIdx.x] = s;
  }
}

// Exclusive scan of sums[0..nb) in place by one block; sums[nb] = total.
__global__ void scan_sums_kernel(int64_t *sums, int nb) {
  __shared__ int64_t tmp[SCAN_THREADS];
  int64_t carry = 0;
  for (int base = 0; base < nb; base += SCAN_THREADS) {
    int i = base + threadIdx.x;
    int64_t v = i < nb ? sums[i] : 0;
    tmp[threadIdx.x] = v;
    __syncthreads();
    for (int d = 1; d < SCAN_THREADS; d <<= 1) {
      int64_t t = threadIdx.x >= d ? tmp[threadIdx.x - d] : 0;
      __syncthreads();
      tmp[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < nb) sums[i] = carry + tmp[threadIdx.x] - v;
    int64_t tot = tmp[SCAN_THREADS - 1];
    __syncthreads();
    carry += tot;
  }
  if (threadIdx.x == 0) sums[nb] = carry;
}

__global__ void block_scan_kernel(int64_t *data, int64_t n, int64_t per_block, const int64_t *sums) {
  __shared__ int64_t tmp[SCAN_THREADS];
  int64_t b0 = blockIdx.x * per_block, b1 = min(n, b0 + per_block);
  int64_t carry = sums[blockIdx.x];
  for (int64_t base = b0; base < b1; base += SCAN_THREADS) {
    int64_t i = base + threadIdx.x;
    int64_t v = i < b1 ? data[i] : 0;
    tmp[threadIdx.x] = v;
    __syncthreads();
    for (int d = 1; d < SCAN_THREADS; d <<= 1) {
      int64_t t = threadIdx.x >= d ? tmp[threadIdx.x - d] : 0;
      __syncthreads();
      tmp[threadIdx.x] += t;
      __syncthreads();
    }
    if (i < b1) data[i] = carry + tmp[threadIdx.x] - v;
    int64_t tot = tmp[SCAN_THREADS - 1];
    __syncthreads();
    carry += tot;
  }
}

__global__ void set_total_kernel(int64_t *data, int64_t n, const int64_t *sums, int nb) {
  data[n] = sums[nb];
}

}  // namespace

// data[0..n) counts -> data[0..n] exclusive offsets, data[n] = total.
// `data` must have room for n + 1 entries.
void exclusive_scan_i64(int64_t *data, int64_t n, cudaStream_t s) {
  int nb = (int)std::min<int64_t>(1024, std::max<int64_t>(1, (n + 65535) / 65536));
  int64_t per_block = (n + nb - 1) / nb;
  DevBuf<int64_t> sums(nb + 1);
  block_sums_kernel<<<nb, SCAN_THREADS, 0, s>>>(data, n, per_block, sums.p);
  scan_sums_kernel<<<1, SCAN_THREADS, 0, s>>>(sums.p, nb);
  block_scan_kernel<<<nb, SCAN_THREADS, 0, s>>>(data, n, per_block, sums.p);
  set_total_kernel<<<1, 1, 0, s>>>(data, n, sums.p, nb);
  RCHOL_CUDA(cudaGetLastError());
  RCHOL_CUDA(cudaStreamSynchronize(s));  // `sums` is freed on return
}

}  // namespace rchol
