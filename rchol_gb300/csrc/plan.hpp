// Triangular-solve schedule of a factor (built once per factor, see trsv.cu).
#pragma once

#include <memory>
#include <mutex>
#include <vector>

#include "common.hpp"

namespace rchol {

// Block stream of one direction (forward with L = G, backward with U = G^T).
//
// The rows of every tree node are cut into pieces that fit in shared memory
// (pieces of one node are solved one after the other) and every piece into
// blocks of 32 consecutive rows.  A piece's entries are
//   * external (columns outside the piece, already solved): a CSR over rows,
//     ext_rp / ext_ci / ext_v, consumed by the prologue;
//   * in an earlier block of the piece: kept sparse in the block's record;
//   * inside the block: folded into the exact inverse of the block's 32x32
//     triangle, stored dense.
// Block record (16-byte aligned, in processing order):
//   u32 nrows, nent, row0 (piece-local first row), col_bytes
//   u32 ent_off[33]                     lane r owns entries [ent_off[r], ent_off[r+1])
//   u16|u32 ent_col[nent]               piece-local columns
//   VT  ent_val[nent]
//   VT  minv[32*32]                     minv[c*32 + r] = (T^-1)_{r,c}
struct NodeDesc {
  int64_t begin;    // first row of the piece
  int32_t rows;
  int32_t nblocks;
  int64_t blk0;     // offsets of its blocks: blk_off[blk0 .. blk0 + nblocks]
  int32_t maxrec;   // largest block record (bytes)
  int32_t wide;     // ent_col is u32 (piece larger than 65535 rows)
};

struct StreamDir {
  std::vector<int> stage_ptr;        // pieces of stage s: [stage_ptr[s], stage_ptr[s+1])
  std::vector<int> stage_split;      // stage uses the multi-block external kernel
  std::vector<int> stage_rows;       // largest piece of the stage (rows)
  std::vector<int> stage_maxrec;     // largest block record of the stage (bytes)
  std::vector<int64_t> stage_row_ptr;  // rows of split stages: srows[stage_row_ptr[s] ..]
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

// Older per-row level schedule, still used for several right-hand sides.
struct DirPlan {
  std::vector<int> stage_ptr;
  std::vector<int> stage_maxrows;
  DevBuf<int64_t> nb, ne;
  DevBuf<int64_t> lvl_off;
  DevBuf<int64_t> level_ptr;
  DevBuf<int32_t> rows;
  DevBuf<int32_t> split;
  int64_t crit_levels = 0;
};

// Workspace and captured CUDA graph of one PCG iteration for a given matrix
// and number of right-hand sides (solve.cu).
struct PcgWork {
  const void *key_rp = nullptr, *key_ci = nullptr, *key_v = nullptr;
  int64_t n = 0, nnz = 0;
  int k = 0;
  DevBuf<double> r, z, p, q, x, sc;
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

struct SolvePlan {
  std::mutex lock;  // solves on one factor are serialised (they share workspaces)
  std::vector<std::unique_ptr<PcgWork>> pcg;
  DirPlan fwd, bwd;
  StreamDir sfwd, sbwd;
  DevBuf<double> dinv;
  DevBuf<float> dinv32;
  int64_t dag_fwd = 0, dag_bwd = 0;
  DevBuf<double> scratch;  // global fallback of the multi-RHS solve
  DevBuf<float> scratch32;
  DevBuf<double> ytmp;     // intermediate of precond (FP64 path)
  DevBuf<float> ytmp32;    // intermediate of precond (FP32 path)
  DevBuf<double> acc64;    // external partial sums of split stages
  DevBuf<float> acc32;
};

void build_streams(const rchol_factor_s &F, SolvePlan &P, cudaStream_t s);
void stream_trsv(const rchol_factor_s &F, const SolvePlan &P, bool upper, const double *in64,
                 const float *in32, double *out64, float *out32, cudaStream_t s);

}  // namespace rchol
