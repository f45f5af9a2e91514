// Triangular-solve schedule of a factor (built once per factor, see trsv.cu).
#pragma once

#include <array>
#include <memory>
#include <mutex>
#include <utility>
#include <vector>

#include "common.hpp"

namespace rchol {

// Block stream of one direction (forward with L = G, backward with U = G^T).
//
// The rows of every tree node are cut into pieces (pieces of one node are
// solved one after another) and every piece into blocks of 32 consecutive
// rows.  A piece's entries are
//   * external (columns outside the piece, already solved): a CSR over rows,
//     ext_rp / ext_ci / ext_v, summed by an all-SM kernel before the stage;
//   * in an earlier block of the piece: kept sparse in the block's record;
//   * inside the block: folded into the exact inverse of the block's 32x32
//     triangle.
// Record formats (trsv.cu documents each): FMT_WARP, one warp per piece with
// a window of solved values (depths with many nodes); FMT_PIPE, one thread
// block per piece whose warps split a block's entries by distance (the few
// long chains at the top of the tree); FMT_KTEAM, a thread block per piece
// for 32 right-hand sides at once.
enum { FMT_WARP = 0, FMT_PIPE = 1, FMT_KTEAM = 2 };

struct NodeDesc {
  int64_t begin;    // first row of the piece
  int32_t rows;
  int32_t nblocks;
  int64_t blk0;     // offsets of its blocks: blk_off[blk0 .. blk0 + nblocks]
  int32_t maxrec;   // largest block record (bytes)
  int32_t wide;     // column indices are u32 (piece larger than 65535 rows)
  int32_t maxchunk; // pipeline / k-team formats: most chunks of one block
  int32_t pad_;
};

struct StreamDir {
  std::vector<int> stage_ptr;        // pieces of stage s: [stage_ptr[s], stage_ptr[s+1])
  std::vector<int> stage_rows;       // largest piece of the stage (rows)
  std::vector<int> stage_maxrec;     // largest block record of the stage (bytes)
  std::vector<int64_t> stage_row_ptr;  // rows of the stages: srows[stage_row_ptr[s] ..]
  std::vector<int> stage_fmt;        // FMT_WARP, FMT_PIPE or FMT_KTEAM
  std::vector<int> stage_warps;      // pipeline / k-team: warps of the stage's teams
  std::vector<int> stage_chunks;     // pipeline / k-team: most chunks of one block in the stage
  std::vector<int> stage_window;     // warp format: rows of the window of solved values (a power of two)
  std::vector<int> stage_ext;        // 1: the stage has external entries (else it reads the rhs directly)
  std::vector<int> stage_ext_lanes;  // lanes per row of the external sums (1, 4, 8 or 32)
  std::vector<std::array<int, 9>> stage_smem;  // pipeline / k-team: launch shared memory by ring depth
  DevBuf<int32_t> srows;
  DevBuf<NodeDesc> nodes;
  DevBuf<int64_t> ext_rp;
  DevBuf<int32_t> ext_ci;
  DevBuf<double> ext_v64;
  DevBuf<float> ext_v32;
  DevBuf<unsigned char> blocks;      // block records (FP32 or FP64 values, per the factor)
  DevBuf<int64_t> blk_off;
  int64_t ext_nnz = 0, sparse_nnz = 0, nblocks = 0;
  int64_t steps = 0;                 // sequential block steps on the critical path
};

// Workspace and captured CUDA graph of one PCG iteration for a given matrix
// and number of right-hand sides (solve.cu).
struct PcgWork {
  uint64_t key_uid = 0;  // the matrix the captured iteration reads
  int64_t n = 0, nnz = 0;
  int k = 0;
  DevBuf<double> r, z, p, q, x, sc;
  DevBuf<double> hb, hx;  // staging of the host-buffer entry point
  DevBuf<int> ic;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t graph_kernels = 0;
  ~PcgWork() {
    if (exec) cudaGraphExecDestroy(exec);
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (stream) cudaStreamDestroy(stream);
  }
};

// Workspace and captured graph of the batched PCG: independent systems that
// are the diagonal blocks (row ranges seg[s] .. seg[s+1]) of one matrix.
struct SegWork {
  uint64_t key_uid = 0;
  std::vector<int64_t> seg_host;
  int64_t n = 0;
  DevBuf<int64_t> seg;
  DevBuf<double> r, z, p, q, x, sc;
  DevBuf<double> hb, hx;
  DevBuf<int> ic;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev_in = nullptr, ev_out = nullptr;
  cudaGraphExec_t exec = nullptr;
  int64_t graph_kernels = 0;
  ~SegWork() {
    if (exec) cudaGraphExecDestroy(exec);
    if (ev_in) cudaEventDestroy(ev_in);
    if (ev_out) cudaEventDestroy(ev_out);
    if (stream) cudaStreamDestroy(stream);
  }
};

// Launch-time choices of the single-right-hand-side solves (trsv.cu).  Any
// setting solves the same system with the same arithmetic; the tuner
// (rchol_gpu_factor_tune) times alternatives on the factor itself.
struct SolveKnobs {
  int pipe_pf = 0;    // pipeline format: records prefetched into L2 ahead of use (0: none)
  int w2_pf = 0;      // warp format: the same
  int pipe_ring = 8;  // pipeline format: most ring slots (5..8)
  int w2_wpb = 8;     // warp format: most warps (pieces) per thread block (1..8)
};

struct SolvePlan {
  std::mutex lock;  // solves on one factor are serialised (they share workspaces)
  SolveKnobs knobs;
  double tuned_ms = 0.0;  // preconditioner time with the tuned knobs (0: not tuned)
  std::vector<std::unique_ptr<PcgWork>> pcg;
  std::vector<std::unique_ptr<SegWork>> seg;
  StreamDir sfwd, sbwd;
  StreamDir kfwd, kbwd;    // pieces for up to 32 right-hand sides (built on first use)
  bool kbuilt = false;
  int64_t dag_fwd = -1, dag_bwd = -1;  // dependency-chain lengths, computed on request
  DevBuf<double> ytmp;     // intermediate of precond (FP64 path)
  DevBuf<float> ytmp32;    // intermediate of precond (FP32 path)
  DevBuf<double> acc64;    // external partial sums of split stages
  DevBuf<float> acc32;
  DevBuf<double> acck64;   // the same for up to 32 right-hand sides (n x 32)
  DevBuf<float> acck32;
};

void build_streams(const rchol_factor_s &F, SolvePlan &P, cudaStream_t s);
void build_streams_k(const rchol_factor_s &F, SolvePlan &P, cudaStream_t s);
// Solve with G (upper = false) or G^T for k right-hand sides, n x k
// row-major, in groups of up to 32 columns.
void stream_trsv_k(const rchol_factor_s &F, const SolvePlan &P, bool upper, const double *in64,
                   const float *in32, double *out64, float *out32, int k, cudaStream_t s);
void stream_trsv(const rchol_factor_s &F, const SolvePlan &P, bool upper, const double *in64,
                 const float *in32, double *out64, float *out32, cudaStream_t s);
// Times the preconditioner under alternative SolveKnobs and keeps the
// fastest; returns {ms with the knobs on entry, ms with the chosen ones}.
std::pair<double, double> tune_solves(const rchol_factor_s &F, SolvePlan &P, cudaStream_t s);

}  // namespace rchol
