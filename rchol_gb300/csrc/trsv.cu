// Block triangular solves with G (forward) and G^T (backward).
//
// Replaces the two MKL trsv calls of c++/util/pcg.cpp:141-159.
//
// Why blocks.  Nested dissection with the reference's natural order inside
// every node leaves long dependency chains (the forward solve at 64^3 has a
// 4,047-row chain; a 4,096-row separator alone has 2,139 levels), so any
// row-by-row or level-by-level schedule is bound by the latency of one step.
// Here the rows of a node are cut into blocks of 32 consecutive rows and each
// block carries the exact inverse of its own 32x32 triangle; one sequential
// step then retires 32 rows instead of one level.
//
// Schedule.  The tree is processed one depth at a time (leaves first for the
// forward solve, root first for the backward one); a node larger than shared
// memory is cut into pieces solved one after another.  Per stage:
//   ext_kernel    acc_i = rhs_i - sum of row i's entries outside its piece
//                 (columns already solved), all SMs; skipped for stages
//                 without such entries (the forward leaves), which read the
//                 right-hand side directly.
//   w2_kernel     depths with many nodes: one warp per piece, many pieces per
//                 SM; lane r sums row r's entries in earlier blocks from a
//                 window of recently solved values, then x = T^-1 t.
//   pipe_kernel   the top of the tree: one thread block per piece whose
//                 warps split each block's entries by distance, so that the
//                 step on the chain (the solver warp) only adds the previous
//                 block's entries and applies the inverse.
// Records stream into shared memory with bulk copies (cp.async.bulk +
// mbarrier); the block inverses are computed in FP64 on the host and rounded
// to the stored precision.  32 right-hand sides at once use the k-team format
// (team_k_kernel).

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <utility>
#include <vector>

#include "common.hpp"
#include "host.hpp"
#include "plan.hpp"

namespace rchol {

namespace {

constexpr int BS = 32;                  // rows per block
constexpr int TRI = BS * (BS + 1) / 2;  // stored entries of a block's triangular inverse

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~size_t(15); }

// Column c of a block inverse is stored contiguously: rows c..31 for a lower
// (forward) inverse, rows 0..c for an upper (backward) one.
__host__ __device__ inline int tri_col_off(int c, bool upper) {
  return upper ? c * (c + 1) / 2 : c * BS - c * (c - 1) / 2;
}

// ---- host: one piece -----------------------------------------------------------

struct PieceBuild {
  std::vector<unsigned char> bytes;  // block records, processing order
  std::vector<int64_t> offs;         // nblocks + 1 relative offsets
  int32_t maxrec = 0;
  int64_t sparse = 0;
};

// Exact inverse of a 32x32 triangular block (rows/cols >= nr are identity).
void invert_block(double T[BS][BS], bool upper, double X[BS][BS]) {
  for (int r = 0; r < BS; ++r)
    for (int c = 0; c < BS; ++c) X[r][c] = 0.0;
  if (!upper) {
    for (int j = 0; j < BS; ++j) {
      X[j][j] = 1.0 / T[j][j];
      for (int i = j + 1; i < BS; ++i) {
        double s = 0.0;
        for (int k = j; k < i; ++k) s += T[i][k] * X[k][j];
        X[i][j] = -s / T[i][i];
      }
    }
  } else {
    for (int j = BS - 1; j >= 0; --j) {
      X[j][j] = 1.0 / T[j][j];
      for (int i = j - 1; i >= 0; --i) {
        double s = 0.0;
        for (int k = i + 1; k <= j; ++k) s += T[i][k] * X[k][j];
        X[i][j] = -s / T[i][i];
      }
    }
  }
}

// Team format.  A thread block of W warps solves the piece: warp 0 (the
// solver) retires one block per step, while the W-1 helper warps prepare the
// block after it: they sum the entries whose columns lie in blocks older than
// the one being solved ("far" entries) in chunks of equal length, one chunk
// per helper thread, reduce the chunks of every row and leave
// u_r = acc_r - far_r for the solver.  The solver adds the previous block's
// entries ("near") with shuffles of the previous block's solution, which it
// still holds in registers, and applies the inverse.  Record (16-byte aligned
// sections):
//   u32 hdr[16]  nrows, row0, prev_row0, nnear, nchunk, chunk_len, col_bytes,
//                nmax (most near entries of one row), then the byte offsets
//                of near_col, near_val, chunk_row, far_col, far_val, minv,
//                near_off
//   near entries, column inside the previous block (0..31) and value, either
//     rows in turn (single right-hand side):
//       u16 near_off[33]; u8 near_col[nnear]; VT near_val[nnear]
//     or slot-major for the 32-wide solve, entry j of row r at j * 32 + r
//     (padding: column 0, value 0):
//       u8 near_col[nmax][32]; VT near_val[nmax][32]
//   u16 chunk_row[33]      row r's chunks [chunk_row[r], chunk_row[r+1])
//   u16|u32 far_col[chunk_len][nchunk]  entry j of chunk c at j * nchunk + c
//   VT  far_val[chunk_len][nchunk]      (padding: column 0, value 0)
//   VT  minv[528]          as in the warp format
// Interleaving the chunks makes the helpers' loads of one step contiguous.
struct TeamLayout {
  size_t o_noff, o_ncol, o_nval, o_crow, o_fcol, o_fval, o_min, len;
};

// nnear: near entries; slots: nmax for the slot-major layout, 0 for rows in turn.
__host__ __device__ inline TeamLayout team_layout(uint32_t nnear, uint32_t slots, uint32_t nchunk, uint32_t clen,
                                                  uint32_t csz, uint32_t vsz) {
  TeamLayout L;
  const size_t nent = slots ? (size_t)BS * slots : nnear;
  L.o_noff = 64;
  L.o_ncol = slots ? 64 : 64 + al16(2 * (BS + 1));
  L.o_nval = L.o_ncol + al16(nent);
  L.o_crow = L.o_nval + al16((size_t)vsz * nent);
  L.o_fcol = L.o_crow + al16(2 * (BS + 1));
  L.o_fval = L.o_fcol + al16((size_t)csz * nchunk * clen);
  L.o_min = L.o_fval + al16((size_t)vsz * nchunk * clen);
  L.len = L.o_min + al16((size_t)vsz * TRI);
  return L;
}

// Upper bound of a team record whose block has `cnt` entries in earlier
// blocks of its piece (near and far entries together), for helpers of
// `helper_threads` threads: chunks of len ceil(cnt / helper_threads) pad at
// most one chunk per row.
inline size_t team_record_bound(size_t cnt, size_t helper_threads, size_t vsz, size_t csz) {
  const size_t slots = helper_threads > (size_t)BS ? helper_threads - BS : 1;
  const size_t clen = std::max<size_t>(1, (cnt + slots - 1) / slots);
  const size_t padded = cnt + BS * clen;
  const size_t near = (size_t)BS * std::min<size_t>(cnt, BS);  // either layout: at most 32 x min(cnt, 32)
  return 64 + al16(2 * (BS + 1)) + al16(near) + al16(vsz * near) + al16(2 * (BS + 1)) + al16(csz * padded) +
         al16(vsz * padded) + al16(vsz * TRI);
}

void build_team_piece(const std::vector<int64_t> &rp, const std::vector<int32_t> &ci, const std::vector<double> &v,
                      int64_t b, int64_t e, bool upper, size_t vsz, int helper_threads, bool slot_major,
                      PieceBuild &P, int32_t &maxchunk) {
  const int64_t R = e - b, nb = (R + BS - 1) / BS;
  const uint32_t csz = R > 65535 ? 4 : 2;
  P.offs.assign(1, 0);
  P.bytes.clear();
  maxchunk = 0;
  double T[BS][BS], X[BS][BS];
  std::vector<std::pair<uint32_t, double>> nearl[BS], farl[BS];
  for (int64_t s = 0; s < nb; ++s) {
    const int64_t bi = upper ? nb - 1 - s : s;
    const int64_t row0 = bi * BS;
    const int nr = (int)std::min<int64_t>(BS, R - row0);
    const int64_t pbi = s == 0 ? -1 : (upper ? bi + 1 : bi - 1);  // previous block, processing order
    const int64_t prow0 = pbi < 0 ? 0 : pbi * BS;
    for (int r = 0; r < BS; ++r) {
      for (int c = 0; c < BS; ++c) T[r][c] = 0.0;
      T[r][r] = 1.0;
      nearl[r].clear();
      farl[r].clear();
    }
    uint32_t nnear = 0, nfar = 0;
    for (int r = 0; r < nr; ++r) {
      const int64_t i = b + row0 + r;
      for (int64_t q = rp[i]; q < rp[i + 1]; ++q) {
        const int64_t c = ci[q];
        if (c < b || c >= e) continue;  // external
        const int64_t lc = c - b, cb = lc / BS;
        if (cb == bi) {
          T[r][lc - row0] = v[q];
        } else if (cb == pbi) {
          nearl[r].push_back({(uint32_t)(lc - prow0), v[q]});
          ++nnear;
        } else {
          farl[r].push_back({(uint32_t)lc, v[q]});
          ++nfar;
        }
      }
    }
    invert_block(T, upper, X);
    // chunks of clen entries (the last one of a row padded), at most one per
    // helper thread (each row adds at most one partial chunk); a chunk never
    // spans two rows
    const int slots = std::max(1, helper_threads - BS);
    const uint32_t clen = std::max<uint32_t>(1, (nfar + slots - 1) / slots);
    uint16_t crow[BS + 1];
    crow[0] = 0;
    uint32_t nchunk = 0, nmax = 0;
    for (int r = 0; r < BS; ++r) {
      nchunk += ((uint32_t)farl[r].size() + clen - 1) / clen;
      crow[r + 1] = (uint16_t)nchunk;
      nmax = std::max<uint32_t>(nmax, (uint32_t)nearl[r].size());
    }
    maxchunk = std::max<int32_t>(maxchunk, (int32_t)nchunk);
    const TeamLayout L = team_layout(nnear, slot_major ? nmax : 0, nchunk, clen, csz, (uint32_t)vsz);
    const size_t base = P.bytes.size();
    P.bytes.resize(base + L.len, 0);
    unsigned char *p = P.bytes.data() + base;
    const uint32_t hdr[16] = {(uint32_t)nr,       (uint32_t)row0,     (uint32_t)prow0,    nnear,
                              nchunk,             clen,               csz,                nmax,
                              (uint32_t)L.o_ncol, (uint32_t)L.o_nval, (uint32_t)L.o_crow, (uint32_t)L.o_fcol,
                              (uint32_t)L.o_fval, (uint32_t)L.o_min,  (uint32_t)L.o_noff, 0};
    std::memcpy(p, hdr, sizeof(hdr));
    auto put_val = [&](size_t off, size_t idx, double x) {
      if (vsz == 8) std::memcpy(p + off + 8 * idx, &x, 8);
      else {
        const float f = (float)x;
        std::memcpy(p + off + 4 * idx, &f, 4);
      }
    };
    uint16_t noff[BS + 1];
    noff[0] = 0;
    size_t w = 0;
    for (int r = 0; r < BS; ++r) {
      for (size_t j = 0; j < nearl[r].size(); ++j, ++w) {
        const size_t at = slot_major ? j * BS + r : w;
        p[L.o_ncol + at] = (unsigned char)nearl[r][j].first;
        put_val(L.o_nval, at, nearl[r][j].second);
      }
      noff[r + 1] = (uint16_t)w;
    }
    // Far entries of chunk c (row r's entries crow[r]*clen.. in column order,
    // clen per chunk), then placed slot by slot.  Helper thread c sums chunk
    // c, so in step j the 32 lanes of a helper warp gather the solved values
    // of slot j of 32 consecutive chunks: within a warp's chunks the entries
    // of each step are chosen greedily so that those gathers hit distinct
    // shared-memory banks where possible (the sum of a chunk does not depend
    // on that order beyond rounding); padding entries (value 0) take a
    // column of a bank that is still free.
    std::vector<std::vector<std::pair<uint32_t, double>>> chunkl(nchunk);
    for (int r = 0; r < BS; ++r)
      for (size_t q = 0; q < farl[r].size(); ++q) chunkl[crow[r] + q / clen].push_back(farl[r][q]);
    const uint32_t nbank = vsz == 4 ? 32 : 16;  // words of one entry of the unknowns
    const int64_t piece_rows = e - b;
    for (uint32_t g0 = 0; g0 < nchunk; g0 += 32) {
      const uint32_t g1 = std::min(nchunk, g0 + 32);
      std::vector<std::vector<char>> taken(g1 - g0);
      for (uint32_t c = g0; c < g1; ++c) taken[c - g0].assign(chunkl[c].size(), 0);
      for (uint32_t j = 0; j < clen; ++j) {
        std::vector<char> busy(nbank, 0);
        std::vector<int> pick(g1 - g0, -1);
        for (uint32_t c = g0; c < g1; ++c) {  // a free bank first, else the first remaining entry
          const auto &lst = chunkl[c];
          int first = -1;
          for (size_t q = 0; q < lst.size(); ++q) {
            if (taken[c - g0][q]) continue;
            if (first < 0) first = (int)q;
            if (!busy[lst[q].first % nbank]) {
              pick[c - g0] = (int)q;
              break;
            }
          }
          if (pick[c - g0] < 0) pick[c - g0] = first;
          if (pick[c - g0] >= 0) {
            taken[c - g0][pick[c - g0]] = 1;
            busy[lst[pick[c - g0]].first % nbank] = 1;
          }
        }
        for (uint32_t c = g0; c < g1; ++c) {
          uint32_t col;
          double val;
          if (pick[c - g0] >= 0) {
            col = chunkl[c][pick[c - g0]].first;
            val = chunkl[c][pick[c - g0]].second;
          } else {  // padding
            uint32_t bank = 0;
            while (bank + 1 < nbank && (busy[bank] || bank >= piece_rows)) ++bank;
            busy[bank] = 1;
            col = bank < piece_rows ? bank : 0;
            val = 0.0;
          }
          const size_t at = (size_t)j * nchunk + c;
          if (csz == 2) {
            const uint16_t c16 = (uint16_t)col;
            std::memcpy(p + L.o_fcol + 2 * at, &c16, 2);
          } else {
            std::memcpy(p + L.o_fcol + 4 * at, &col, 4);
          }
          put_val(L.o_fval, at, val);
        }
      }
    }
    if (!slot_major) std::memcpy(p + L.o_noff, noff, sizeof(noff));
    std::memcpy(p + L.o_crow, crow, sizeof(crow));
    for (int c = 0; c < BS; ++c) {
      const int r_lo = upper ? 0 : c, r_hi = upper ? c : BS - 1;
      for (int r = r_lo; r <= r_hi; ++r)
        put_val(L.o_min, (size_t)tri_col_off(c, upper) + (size_t)(r - r_lo), (r < nr && c < nr) ? X[r][c] : 0.0);
    }
    P.offs.push_back((int64_t)P.bytes.size());
    P.maxrec = std::max<int32_t>(P.maxrec, (int32_t)L.len);
    P.sparse += nnear + nfar;
  }
}

// ---- device ----------------------------------------------------------------------

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
  unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

#ifdef RCHOL_DEVICE_CHECKS
// Diagnostic build only: bounds checks report the first violations and skip
// the access (uniform conditions make the whole warp leave).
__device__ int64_t dbg_n;
__device__ unsigned dbg_count;
__device__ void dbg_report(const char *what, int64_t v, int64_t lim) {
  if (atomicAdd(&dbg_count, 1u) < 16u)
    printf("[rchol check] %s: %lld (limit %lld) block %d thread %d\n", what, (long long)v, (long long)lim,
           (int)blockIdx.x, (int)threadIdx.x);
}
#endif

// acc_i = rhs_i - sum over row i's entries outside its piece.
template <typename VT, typename InT, typename OutT>
__global__ void __launch_bounds__(256) ext_kernel(const int32_t *__restrict__ rows, int64_t nrows,
                                                  const int64_t *__restrict__ ext_rp, const int32_t *__restrict__ ext_ci,
                                                  const VT *__restrict__ ext_v, const InT *__restrict__ in,
                                                  const OutT *out, VT *__restrict__ acc) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  const int64_t i = rows[t];
#ifdef RCHOL_DEVICE_CHECKS
  if (i < 0 || i >= dbg_n) {
    dbg_report("ext row", i, dbg_n);
    return;
  }
#endif
  const int64_t q0 = ext_rp[i], q1 = ext_rp[i + 1];
  VT s0 = 0, s1 = 0;
  int64_t q = q0;
#ifdef RCHOL_DEVICE_CHECKS
  for (int64_t qq = q0; qq < q1; ++qq)
    if (ext_ci[qq] < 0 || ext_ci[qq] >= dbg_n) {
      dbg_report("ext col", ext_ci[qq], dbg_n);
      return;
    }
#endif
  for (; q + 1 < q1; q += 2) {
    s0 += ext_v[q] * (VT)out[ext_ci[q]];
    s1 += ext_v[q + 1] * (VT)out[ext_ci[q + 1]];
  }
  if (q < q1) s0 += ext_v[q] * (VT)out[ext_ci[q]];
  acc[i] = (VT)in[i] - (s0 + s1);
}

// acc_i = rhs_i - sum over row i's entries outside its piece, LANES lanes per
// row (long external rows at the top of the tree); fixed summation order.
template <typename VT, typename InT, typename OutT, int LANES>
__global__ void __launch_bounds__(256) ext_lanes_kernel(const int32_t *__restrict__ rows, int64_t nrows,
                                                        const int64_t *__restrict__ ext_rp,
                                                        const int32_t *__restrict__ ext_ci,
                                                        const VT *__restrict__ ext_v, const InT *__restrict__ in,
                                                        const OutT *out, VT *__restrict__ acc) {
  const int64_t t = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) / LANES;
  const int sub = threadIdx.x % LANES;
  if (t >= nrows) return;  // whole groups leave together (LANES divides 32)
  const int64_t i = rows[t];
  const int64_t q1 = ext_rp[i + 1];
  VT s0 = 0, s1 = 0;
  int64_t q = ext_rp[i] + sub;
  for (; q + LANES < q1; q += 2 * LANES) {
    s0 += ext_v[q] * (VT)out[ext_ci[q]];
    s1 += ext_v[q + LANES] * (VT)out[ext_ci[q + LANES]];
  }
  if (q < q1) s0 += ext_v[q] * (VT)out[ext_ci[q]];
  VT s = s0 + s1;
  const unsigned mask = LANES == 32 ? 0xffffffffu : (((1u << LANES) - 1u) << ((threadIdx.x & 31) / LANES * LANES));
#pragma unroll
  for (int o = LANES / 2; o; o >>= 1) s += __shfl_xor_sync(mask, s, o, LANES);
  if (sub == 0) acc[i] = (VT)in[i] - s;
}

// Status of the solve kernels, read and cleared by the host
// (take_solve_status): bit 0, a bounded wait gave up; bit 1, a piece did not
// fit its launch's shared memory.
__device__ unsigned int g_solve_status;

template <typename VT>
struct TeamArgs {
  const NodeDesc *nodes;
  int node0;            // first piece of the stage; piece = node0 + blockIdx.x
  int smem;             // dynamic shared memory of the launch (bytes)
  int ring;             // most records in the ring (3..8): the solved block's, the next one's, ring-2 in flight
  int maxchunk;         // most chunks of one block (chunk-sum buffer)
  const unsigned char *blocks;
  const int64_t *blk_off;
  const VT *acc;
};

constexpr int TEAM_RING = 4;  // ring used to cut pieces; launches deepen it where room is left
constexpr int TEAM_RING_MIN = 3;
constexpr int TEAM_RING_MAX = 8;

// cp.async.wait_group takes an immediate: wait until at most n groups pend.
__device__ __forceinline__ void cp_async_wait_upto(int n) {
  switch (n) {
    case 0: cp_async_wait<0>(); break;
    case 1: cp_async_wait<1>(); break;
    case 2: cp_async_wait<2>(); break;
    case 3: cp_async_wait<3>(); break;
    case 4: cp_async_wait<4>(); break;
    default: cp_async_wait<5>(); break;
  }
}

// Header of a team record, read with four 16-byte loads.
struct TeamHdr {
  uint32_t nr, row0, prow0, nnear, nchunk, clen, csz, nmax;
  uint32_t o_ncol, o_nval, o_crow, o_fcol, o_fval, o_min, o_noff, pad;
};

__device__ __forceinline__ TeamHdr read_hdr(const unsigned char *p) {
  const uint4 *q = reinterpret_cast<const uint4 *>(p);
  const uint4 a = q[0], b = q[1], c = q[2], d = q[3];
  return TeamHdr{a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w, c.x, c.y, c.z, c.w, d.x, d.y, d.z, d.w};
}

// ---- several right-hand sides -----------------------------------------------------
//
// Vectors are n x ld row-major; one pass solves k <= KW consecutive columns
// (acc is n x KW).  Lane j of a warp owns right-hand
// side j, so every entry of G is read once for all k and applied with one
// FMA per lane; the piece's unknowns sit in shared memory as rows of KW
// values.  The records are the team format's, in pieces cut for KW-wide rows.

constexpr int KW = 32;

template <typename VT, typename InT, typename OutT>
__global__ void __launch_bounds__(256) ext_k_kernel(const int32_t *__restrict__ rows, int64_t nrows,
                                                   const int64_t *__restrict__ ext_rp,
                                                   const int32_t *__restrict__ ext_ci, const VT *__restrict__ ext_v,
                                                   const InT *__restrict__ in, const OutT *out,
                                                   VT *__restrict__ acc, int k, int64_t ld) {
  const int64_t t = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= nrows || lane >= k) return;
  const int64_t i = rows[t];
  const int64_t q1 = ext_rp[i + 1];
  VT s0 = 0, s1 = 0;
  int64_t q = ext_rp[i];
  for (; q + 1 < q1; q += 2) {
    s0 += ext_v[q] * (VT)out[(int64_t)ext_ci[q] * ld + lane];
    s1 += ext_v[q + 1] * (VT)out[(int64_t)ext_ci[q + 1] * ld + lane];
  }
  if (q < q1) s0 += ext_v[q] * (VT)out[(int64_t)ext_ci[q] * ld + lane];
  acc[i * KW + lane] = (VT)in[i * ld + lane] - (s0 + s1);
}

// One thread block per piece.  Warp 0 solves block b for all right-hand sides
// (t = acc - near - far sums, x = T^-1 t with the packed inverse, in
// registers); helper warps sum the far entries of block b+1 row by row into
// part[(b+1)&1][row][lane] and stream the records.  One barrier per block.
template <typename VT, typename OutT, bool UPPER>
__global__ void __launch_bounds__(256, 1) team_k_kernel(TeamArgs<VT> a, OutT *out, int k, int64_t ld) {
  extern __shared__ __align__(16) unsigned char smem[];
  const NodeDesc nd = a.nodes[a.node0 + blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ht = tid - 32, TH = (int)blockDim.x - 32, HW = (int)(blockDim.x >> 5) - 1;
  // this piece's ring: records of its longest, as many (up to a.ring) as the
  // launch's shared memory holds besides the chunk sums and its rows
  const size_t bufbytes = al16((size_t)nd.maxrec);
  const size_t fixed = 2 * (size_t)BS * KW * sizeof(VT) + (size_t)nd.rows * KW * sizeof(VT);
  const int RING = min(a.ring, (int)(((size_t)a.smem - min((size_t)a.smem, fixed)) / bufbytes));
  if (RING < TEAM_RING_MIN) {  // excluded by the plan (every piece fits the smallest ring)
    if (tid == 0) atomicOr(&g_solve_status, 2u);
    return;
  }
  unsigned char *ring = smem;
  VT *part = reinterpret_cast<VT *>(smem + (size_t)RING * bufbytes);  // [2][BS][KW]
  VT *xs = part + 2 * BS * KW;                                           // [rows][KW]
  const unsigned char *src = a.blocks;
  const int64_t *boff = a.blk_off + nd.blk0;
  const int nb = nd.nblocks;

  auto load = [&](int b) {
    if (b < nb) {
      unsigned char *dst = ring + (size_t)(b % RING) * bufbytes;
      const int64_t o0 = boff[b], len = boff[b + 1] - o0;
      for (int64_t o = (int64_t)ht * 16; o < len; o += (int64_t)TH * 16) cp_async16(dst + o, src + o0 + o);
    }
    cp_async_commit();
  };
  for (int idx = tid; idx < nd.rows * KW; idx += blockDim.x) {
    const int r = idx / KW, j = idx % KW;
    xs[idx] = j < k ? a.acc[(nd.begin + r) * (int64_t)KW + j] : VT(0);
  }
  for (int idx = tid; idx < 2 * BS * KW; idx += blockDim.x) part[idx] = VT(0);  // block 0 has no far sums
  if (warp > 0) {
    for (int b = 0; b < RING - 1; ++b) load(b);
    cp_async_wait_upto(RING - 3);
  }
  __syncthreads();

  for (int b = 0; b < nb; ++b) {
    if (warp == 0) {
      const unsigned char *p = ring + (size_t)(b % RING) * bufbytes;
      const TeamHdr h = read_hdr(p);
      const uint32_t nr = h.nr, row0 = h.row0, prow0 = h.prow0;
      const unsigned char *ncol = p + h.o_ncol;
      const VT *nval = reinterpret_cast<const VT *>(p + h.o_nval);
      const VT *minv = reinterpret_cast<const VT *>(p + h.o_min);
      const VT *pb = part + (size_t)(b & 1) * BS * KW;
      VT t[BS];
#pragma unroll
      for (int r = 0; r < BS; ++r) t[r] = r < (int)nr ? xs[(row0 + r) * KW + lane] - pb[r * KW + lane] : VT(0);
      // near entries, slot by slot: the 32 rows of a slot are independent
      for (uint32_t j = 0; j < h.nmax; ++j) {
#pragma unroll
        for (int r = 0; r < BS; ++r)
          t[r] -= nval[j * BS + r] * xs[(prow0 + ncol[j * BS + r]) * KW + lane];
      }
#pragma unroll
      for (int r = 0; r < BS; ++r)
        if (r >= (int)nr) t[r] = VT(0);
      // x = T^-1 t in place: lower rows from the last up, upper from the first down
#pragma unroll
      for (int i = 0; i < BS; ++i) {
        const int r = UPPER ? i : BS - 1 - i;
        VT s = 0;
#pragma unroll
        for (int c = UPPER ? r : 0; c <= (UPPER ? BS - 1 : r); ++c)
          s += minv[tri_col_off(c, UPPER) + (UPPER ? r : r - c)] * t[c];
        t[r] = s;
      }
#pragma unroll
      for (int r = 0; r < BS; ++r)
        if (r < (int)nr) xs[(row0 + r) * KW + lane] = t[r];
    } else {
      if (b + 1 < nb) {
        const unsigned char *p = ring + (size_t)((b + 1) % RING) * bufbytes;
        const TeamHdr h = read_hdr(p);
        const uint32_t csz = h.csz;
        const uint16_t *crow = reinterpret_cast<const uint16_t *>(p + h.o_crow);
        const VT *fval = reinterpret_cast<const VT *>(p + h.o_fval);
        VT *pb = part + (size_t)((b + 1) & 1) * BS * KW;
        const uint32_t nch = h.nchunk, clen = h.clen;
        for (int r = warp - 1; r < BS; r += HW) {
          VT s0 = 0, s1 = 0;
          for (uint32_t c = crow[r]; c < crow[r + 1]; ++c) {  // the row's chunks, entries strided by nchunk
            if (csz == 2) {
              const uint16_t *col = reinterpret_cast<const uint16_t *>(p + h.o_fcol);
              for (uint32_t j = 0, at = c; j < clen; ++j, at += nch) {
                const VT v = fval[at] * xs[col[at] * KW + lane];
                if (j & 1) s1 += v;
                else s0 += v;
              }
            } else {
              const uint32_t *col = reinterpret_cast<const uint32_t *>(p + h.o_fcol);
              for (uint32_t j = 0, at = c; j < clen; ++j, at += nch) {
                const VT v = fval[at] * xs[(size_t)col[at] * KW + lane];
                if (j & 1) s1 += v;
                else s0 += v;
              }
            }
          }
          pb[r * KW + lane] = s0 + s1;
        }
      }
      load(b + RING - 1);
      cp_async_wait_upto(RING - 3);
    }
    __syncthreads();
  }
  for (int idx = tid; idx < nd.rows * KW; idx += blockDim.x) {
    const int r = idx / KW, j = idx % KW;
    if (j < k) out[(nd.begin + r) * ld + j] = (OutT)xs[idx];
  }
}

// ---- single right-hand side: the packed block inverse ---------------------------------
//
// Row r of a block's inverse is stored by quads of 4 values: columns 0..r of
// a lower (forward) inverse in quads 0..r/4, columns r..31 of an upper
// (backward) one in quads r/4..7, zero-padded inside the end quads.  The
// lane that owns row r loads its row with at most eight 16-byte reads and
// multiplies it with the block's right-hand side t, which every lane reads
// from shared memory as the same eight quads (broadcast reads).
constexpr int TQ = 144;  // quads of one packed inverse (576 values)

__host__ __device__ inline int tq_lo(int r, bool upper) { return upper ? (r >> 2) : 0; }
__host__ __device__ inline int tq_hi(int r, bool upper) { return upper ? 7 : (r >> 2); }
// first quad of row r: sum over earlier rows of their quad counts
__host__ __device__ inline int tq_off(int r, bool upper) {
  const int q = r >> 2, m = r & 3;
  return upper ? 8 * r - 2 * q * (q - 1) - m * q : 2 * q * (q + 1) + m * (q + 1);
}

inline void put_val(unsigned char *p, size_t vsz, size_t idx, double x) {
  if (vsz == 8) std::memcpy(p + 8 * idx, &x, 8);
  else {
    const float f = (float)x;
    std::memcpy(p + 4 * idx, &f, 4);
  }
}

// X: the inverse of the block's triangle (rows/columns >= nr unused).
void put_tinv(unsigned char *p, size_t vsz, const double X[BS][BS], int nr, bool upper) {
  for (int r = 0; r < BS; ++r)
    for (int q = tq_lo(r, upper); q <= tq_hi(r, upper); ++q)
      for (int j = 0; j < 4; ++j) {
        const int c = 4 * q + j;
        const bool in = upper ? c >= r : c <= r;
        put_val(p, vsz, 4 * (size_t)(tq_off(r, upper) + q - tq_lo(r, upper)) + j,
                (in && r < nr && c < nr) ? X[r][c] : 0.0);
      }
}

// ---- warp format: one warp per piece -------------------------------------------------
//
// Lane r owns row r of a block: it sums the row's entries in earlier blocks
// of the piece (already solved) and applies the inverse.  The piece's solved
// values live in a window of W rows of shared memory (row i at i mod W): the
// planner picks W above the longest distance between a row and the columns
// it reads, so nodes of thousands of rows whose entries stay near the
// diagonal (the leaves) need only a few KB.  Record (16-byte sections):
//   u32 hdr[4]        nrows, row0, nent, col_bytes
//   u16 eoff[33]      row r's entries [eoff[r], eoff[r+1])
//   u16|u32 col[nent] piece-local columns
//   VT  val[nent]
//   VT  tinv[576]     packed inverse
struct W2Layout {
  size_t o_eoff, o_col, o_val, o_tinv, len;
};

__host__ __device__ inline W2Layout w2_layout(uint32_t nent, uint32_t csz, uint32_t vsz) {
  W2Layout L;
  L.o_eoff = 16;
  L.o_col = 16 + al16(2 * (BS + 1));
  L.o_val = L.o_col + al16((size_t)csz * nent);
  L.o_tinv = L.o_val + al16((size_t)vsz * nent);
  L.len = L.o_tinv + (size_t)vsz * 4 * TQ;
  return L;
}

inline size_t w2_record_bound(size_t cnt, size_t vsz, size_t csz) {
  return 16 + al16(2 * (BS + 1)) + al16(csz * cnt) + al16(vsz * cnt) + vsz * 4 * TQ;
}

// Records of one warp-format piece; `reach` returns the longest distance
// (in rows) between a row and a column it reads inside the piece.
void build_w2_piece(const std::vector<int64_t> &rp, const std::vector<int32_t> &ci, const std::vector<double> &v,
                    int64_t b, int64_t e, bool upper, size_t vsz, PieceBuild &P, int64_t &reach) {
  const int64_t R = e - b, nb = (R + BS - 1) / BS;
  const uint32_t csz = R > 65535 ? 4 : 2;
  P.offs.assign(1, 0);
  P.bytes.clear();
  reach = 0;
  double T[BS][BS], X[BS][BS];
  std::vector<uint32_t> cols[BS];
  std::vector<double> vals[BS];
  for (int64_t s = 0; s < nb; ++s) {
    const int64_t bi = upper ? nb - 1 - s : s;
    const int64_t row0 = bi * BS;
    const int nr = (int)std::min<int64_t>(BS, R - row0);
    for (int r = 0; r < BS; ++r) {
      for (int c = 0; c < BS; ++c) T[r][c] = 0.0;
      T[r][r] = 1.0;
      cols[r].clear();
      vals[r].clear();
    }
    uint32_t nent = 0;
    for (int r = 0; r < nr; ++r) {
      const int64_t i = b + row0 + r;
      for (int64_t q = rp[i]; q < rp[i + 1]; ++q) {
        const int64_t c = ci[q];
        if (c < b || c >= e) continue;  // external
        const int64_t lc = c - b;
        reach = std::max<int64_t>(reach, std::abs(row0 + r - lc));
        if (lc >= row0 && lc < row0 + nr) {
          T[r][lc - row0] = v[q];
        } else {
          cols[r].push_back((uint32_t)lc);
          vals[r].push_back(v[q]);
          ++nent;
        }
      }
    }
    if (nent > 65535) throw Error(RCHOL_ERR_INTERNAL, "a 32-row block has too many entries for the warp format");
    invert_block(T, upper, X);
    const W2Layout L = w2_layout(nent, csz, (uint32_t)vsz);
    const size_t base = P.bytes.size();
    P.bytes.resize(base + L.len, 0);
    unsigned char *p = P.bytes.data() + base;
    const uint32_t hdr[4] = {(uint32_t)nr, (uint32_t)row0, nent, csz};
    std::memcpy(p, hdr, 16);
    uint16_t eoff[BS + 1];
    eoff[0] = 0;
    size_t w = 0;
    for (int r = 0; r < BS; ++r) {
      for (size_t t = 0; t < cols[r].size(); ++t, ++w) {
        if (csz == 2) {
          const uint16_t c16 = (uint16_t)cols[r][t];
          std::memcpy(p + L.o_col + 2 * w, &c16, 2);
        } else {
          std::memcpy(p + L.o_col + 4 * w, &cols[r][t], 4);
        }
        put_val(p + L.o_val, vsz, w, vals[r][t]);
      }
      eoff[r + 1] = (uint16_t)w;
    }
    std::memcpy(p + L.o_eoff, eoff, sizeof(eoff));
    put_tinv(p + L.o_tinv, vsz, X, nr, upper);
    P.offs.push_back((int64_t)P.bytes.size());
    P.maxrec = std::max<int32_t>(P.maxrec, (int32_t)L.len);
    P.sparse += nent;
  }
}

// ---- pipeline format: one thread block per piece --------------------------------------
//
// For the few long chains at the top of the tree.  With t = acc - (entries in
// earlier blocks)·x and N1 / N2 / F the block's entries in the previous block,
// the one before and older ones,
//   x_k = T^-1 t = w_k + y_k - P_k x_{k-1},
//   w_k = T^-1 (acc_k - F_k x),  y_k = -Q_k x_{k-2},  P = T^-1 N1,  Q = T^-1 N2,
// with P and Q computed in FP64 on the host.  Each term is prepared by its
// own warp as soon as its inputs exist, so the chain of the solver warp in
// step k is one shared-memory read (w + y) and 32 FMAs with P's row and
// x_{k-1}, both already in its registers.
// Record (16-byte sections):
//   u32 hdr[16]  nrows, row0, prow0, pprow0, nchunk, clen, col_bytes, o_crow,
//                o_fc, o_fv, stride (P / Q row stride in values), 0...
//   VT  tinv[576]                 packed inverse (at byte 64), the reducer's
//   VT  P[32][stride], Q[32][stride]  dense, rows padded (conflict-free
//                                 16-byte row reads by 32 lanes)
//   u16 crow[33]                  row r's chunks [crow[r], crow[r+1])
//   u16|u32 fc[clen][nchunk]; VT fv[..]  far entries, entry j of chunk c at j*nchunk + c
__host__ __device__ constexpr int pq_stride(size_t vsz) { return vsz == 4 ? 36 : 34; }
// byte offset of crow: fixed by the value size
__host__ __device__ constexpr size_t pipe_o_crow(size_t vsz) { return 64 + vsz * 4 * TQ + 2 * vsz * BS * pq_stride(vsz); }
constexpr int kPipeRoleWarps = 4;  // solver, reducer, mixer, record streamer; the other warps of a team gather
constexpr int kPipeRingCut = 6;  // ring the pieces are cut for (launch: up to kPipeRingMax)
constexpr int kPipeRingMin = 5;  // records k+1..k+3 in use, k+4 waited for, one in flight
constexpr int kPipeRingMax = 8;
// most chunks of one row's far entries: FP32 16 (two batches of the
// reducer's loads, shorter gatherer chunks), FP64 8 (one batch; measured
// 12% faster than 16 for FP64, 1-3% slower for FP32)
inline uint32_t pipe_row_chunks(size_t vsz) { return vsz == 4 ? 16u : 8u; }

struct PipeLayout {
  size_t o_tinv, o_p, o_q, o_crow, o_fc, o_fv, len;
};

__host__ __device__ inline PipeLayout pipe_layout(uint32_t nchunk, uint32_t clen, uint32_t csz, uint32_t vsz) {
  PipeLayout L;
  const size_t pq = (size_t)vsz * BS * pq_stride(vsz);
  L.o_tinv = 64;
  L.o_p = L.o_tinv + (size_t)vsz * 4 * TQ;
  L.o_q = L.o_p + pq;
  L.o_crow = L.o_q + pq;  // == pipe_o_crow(vsz)
  L.o_fc = L.o_crow + al16(2 * (BS + 1));
  L.o_fv = L.o_fc + al16((size_t)csz * nchunk * clen);
  L.len = L.o_fv + al16((size_t)vsz * nchunk * clen);
  return L;
}

// Chunking of a pipeline record's far entries (`rf[r]` of row r, `nfar` in
// all): chunks of clen entries (a row's last chunk padded), one chunk per
// gatherer thread (every row adds at most one partial chunk, so
// ceil(nfar / (gthreads - 32)) entries per chunk suffice), and no row in more
// than pipe_row_chunks(vsz) chunks, so that the reducer's lane for a row sums
// its chunks in one or two batches of loads.
struct PipeChunks {
  uint32_t clen, nchunk;
};
inline PipeChunks pipe_chunks(const uint32_t *rf, uint32_t nfar, int gthreads, size_t vsz) {
  const uint32_t slots = (uint32_t)std::max(1, gthreads - BS), rc = pipe_row_chunks(vsz);
  uint32_t longest = 0;
  for (int r = 0; r < BS; ++r) longest = std::max(longest, rf[r]);
  PipeChunks c;
  c.clen = std::max<uint32_t>({1u, (nfar + slots - 1) / slots, (longest + rc - 1) / rc});
  c.nchunk = 0;
  for (int r = 0; r < BS; ++r) c.nchunk += (rf[r] + c.clen - 1) / c.clen;
  return c;
}

// Length of a pipeline record whose rows have `rf[r]` entries more than two
// blocks back in their piece, for `gthreads` gatherer threads.
inline size_t pipe_record_len(const uint32_t *rf, uint32_t nfar, int gthreads, size_t vsz, size_t csz) {
  const PipeChunks c = pipe_chunks(rf, nfar, gthreads, vsz);
  return pipe_layout(c.nchunk, c.clen, (uint32_t)csz, (uint32_t)vsz).len;
}

void build_pipe_piece(const std::vector<int64_t> &rp, const std::vector<int32_t> &ci, const std::vector<double> &v,
                      int64_t b, int64_t e, bool upper, size_t vsz, int gthreads, PieceBuild &P,
                      int32_t &maxchunk) {
  const int64_t R = e - b, nb = (R + BS - 1) / BS;
  const uint32_t csz = R > 65535 ? 4 : 2;
  const int stride = pq_stride(vsz);
  P.offs.assign(1, 0);
  P.bytes.clear();
  maxchunk = 0;
  double T[BS][BS], X[BS][BS], N1[BS][BS], N2[BS][BS];
  std::vector<std::pair<uint32_t, double>> lf[BS];
  for (int64_t s = 0; s < nb; ++s) {
    const int64_t bi = upper ? nb - 1 - s : s;
    const int64_t row0 = bi * BS;
    const int nr = (int)std::min<int64_t>(BS, R - row0);
    const int64_t b1 = upper ? bi + 1 : bi - 1, b2 = upper ? bi + 2 : bi - 2;  // blocks k-1, k-2
    const bool has1 = s >= 1, has2 = s >= 2;
    for (int r = 0; r < BS; ++r) {
      for (int c = 0; c < BS; ++c) T[r][c] = N1[r][c] = N2[r][c] = 0.0;
      T[r][r] = 1.0;
      lf[r].clear();
    }
    uint32_t nfar = 0;
    for (int r = 0; r < nr; ++r) {
      const int64_t i = b + row0 + r;
      for (int64_t q = rp[i]; q < rp[i + 1]; ++q) {
        const int64_t c = ci[q];
        if (c < b || c >= e) continue;  // external
        const int64_t lc = c - b, cb = lc / BS;
        if (cb == bi) T[r][lc - row0] = v[q];
        else if (has1 && cb == b1) N1[r][lc - b1 * BS] = v[q];
        else if (has2 && cb == b2) N2[r][lc - b2 * BS] = v[q];
        else {
          lf[r].push_back({(uint32_t)lc, v[q]});
          ++nfar;
        }
      }
    }
    invert_block(T, upper, X);
    uint32_t rf[BS];
    for (int r = 0; r < BS; ++r) rf[r] = (uint32_t)lf[r].size();
    const PipeChunks pc = pipe_chunks(rf, nfar, gthreads, vsz);
    const uint32_t clen = pc.clen, nchunk = pc.nchunk;
    uint16_t crow[BS + 1];
    crow[0] = 0;
    for (int r = 0; r < BS; ++r) crow[r + 1] = (uint16_t)(crow[r] + (rf[r] + clen - 1) / clen);
    if (nchunk > (uint32_t)gthreads) throw Error(RCHOL_ERR_INTERNAL, "pipeline record: more chunks than gatherers");
    maxchunk = std::max<int32_t>(maxchunk, (int32_t)nchunk);
    const PipeLayout L = pipe_layout(nchunk, clen, csz, (uint32_t)vsz);
    if (L.o_crow != pipe_o_crow(vsz)) throw Error(RCHOL_ERR_INTERNAL, "pipeline record: crow offset");
    const size_t base = P.bytes.size();
    P.bytes.resize(base + L.len, 0);
    unsigned char *p = P.bytes.data() + base;
    const int64_t prow0 = has1 ? b1 * BS : 0, pprow0 = has2 ? b2 * BS : 0;
    const uint32_t hdr[16] = {(uint32_t)nr,      (uint32_t)row0,    (uint32_t)prow0,  (uint32_t)pprow0,
                              nchunk,            clen,              csz,              (uint32_t)L.o_crow,
                              (uint32_t)L.o_fc,  (uint32_t)L.o_fv,  (uint32_t)stride, 0,
                              0,                 0,                 0,                0};
    std::memcpy(p, hdr, sizeof(hdr));
    put_tinv(p + L.o_tinv, vsz, X, nr, upper);
    // P = T^-1 N1, Q = T^-1 N2 (rows and columns beyond the block's rows are zero)
    for (int r = 0; r < BS; ++r)
      for (int c = 0; c < BS; ++c) {
        double pr = 0.0, qr = 0.0;
        if (r < nr)
          for (int k = 0; k < nr; ++k) {
            const double t = X[r][k];
            if (t == 0.0) continue;
            pr += t * N1[k][c];
            qr += t * N2[k][c];
          }
        put_val(p + L.o_p, vsz, (size_t)r * stride + c, pr);
        put_val(p + L.o_q, vsz, (size_t)r * stride + c, qr);
      }
    std::memcpy(p + L.o_crow, crow, sizeof(crow));
    // chunk c holds row r's far entries crow[r]*clen.. in column order; within
    // each warp's 32 chunks the entries of one step are picked greedily so that
    // the gathers of the solved values hit distinct shared-memory banks where
    // possible (the chunk's sum does not depend on that order beyond
    // rounding); padding entries (value 0) take a column of a free bank
    std::vector<std::vector<std::pair<uint32_t, double>>> chunkl(nchunk);
    for (int r = 0; r < BS; ++r)
      for (size_t q = 0; q < lf[r].size(); ++q) chunkl[crow[r] + q / clen].push_back(lf[r][q]);
    const uint32_t nbank = vsz == 4 ? 32 : 16;
    for (uint32_t g0 = 0; g0 < nchunk; g0 += 32) {
      const uint32_t g1 = std::min(nchunk, g0 + 32);
      std::vector<std::vector<char>> taken(g1 - g0);
      for (uint32_t c = g0; c < g1; ++c) taken[c - g0].assign(chunkl[c].size(), 0);
      for (uint32_t j = 0; j < clen; ++j) {
        std::vector<char> busy(nbank, 0);
        std::vector<int> pick(g1 - g0, -1);
        for (uint32_t c = g0; c < g1; ++c) {
          const auto &lst = chunkl[c];
          int first = -1;
          for (size_t q = 0; q < lst.size(); ++q) {
            if (taken[c - g0][q]) continue;
            if (first < 0) first = (int)q;
            if (!busy[lst[q].first % nbank]) {
              pick[c - g0] = (int)q;
              break;
            }
          }
          if (pick[c - g0] < 0) pick[c - g0] = first;
          if (pick[c - g0] >= 0) {
            taken[c - g0][pick[c - g0]] = 1;
            busy[lst[pick[c - g0]].first % nbank] = 1;
          }
        }
        for (uint32_t c = g0; c < g1; ++c) {
          uint32_t col;
          double val;
          if (pick[c - g0] >= 0) {
            col = chunkl[c][pick[c - g0]].first;
            val = chunkl[c][pick[c - g0]].second;
          } else {  // padding
            uint32_t bank = 0;
            while (bank + 1 < nbank && (busy[bank] || bank >= R)) ++bank;
            busy[bank] = 1;
            col = bank < R ? bank : 0;
            val = 0.0;
          }
          const size_t at = (size_t)j * nchunk + c;
          if (csz == 2) {
            const uint16_t c16 = (uint16_t)col;
            std::memcpy(p + L.o_fc + 2 * at, &c16, 2);
          } else {
            std::memcpy(p + L.o_fc + 4 * at, &col, 4);
          }
          put_val(p + L.o_fv, vsz, at, val);
        }
      }
    }
    P.offs.push_back((int64_t)P.bytes.size());
    P.maxrec = std::max<int32_t>(P.maxrec, (int32_t)L.len);
    P.sparse += nfar;
    for (int r = 0; r < BS; ++r)
      for (int c = 0; c < BS; ++c) P.sparse += (N1[r][c] != 0.0) + (N2[r][c] != 0.0);
  }
}

// ---- bulk copies into shared memory ----------------------------------------------------
//
// Records stream into a ring of shared-memory slots with cp.async.bulk (the
// copy engine moves a whole record; no thread issues 16-byte pieces), one
// mbarrier per slot counting the record's bytes.  Far-ahead records are
// prefetched into L2.  Every wait is bounded: after kWaitLimit polls the
// kernel records bit 0 in g_solve_status, stops issuing copies, waits
// (bounded) for the ones in flight and finishes without using the data.

constexpr uint32_t kWaitLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
// orders this thread's earlier shared-memory accesses before later async-proxy (bulk copy) ones
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(bar))
               : "memory");
}
__device__ __forceinline__ void prefetch_l2(const void *src, uint32_t bytes) {
  asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;\n" ::"l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_test(uint64_t *bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_addr(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase of `parity` to complete; false after kWaitLimit polls.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (uint32_t i = 0; i < kWaitLimit; ++i)
    if (mbar_test(bar, parity)) return true;
  return false;
}

// Byte offsets of a piece's records, held by the 32 lanes of one warp: lane j
// has boff[32c + j] (window A) and boff[32c + 32 + j] (window B); get(k) is a
// warp-wide shuffle and valid for 32c <= k < 32c + 64.  advance(k) slides the
// windows once k reaches 32c + 32, loading the next 32 offsets about 32
// records before they are needed (offsets past the end read the last one).
struct OffCache {
  const int64_t *boff;
  int last;  // index of the last offset (= number of records)
  int c32;   // 32c
  int64_t a, b;
  __device__ void init(const int64_t *p, int nrec, int lane) {
    boff = p;
    last = nrec;
    c32 = 0;
    a = boff[min(lane, last)];
    b = boff[min(32 + lane, last)];
  }
  __device__ __forceinline__ int64_t get(int k) const {
    const int64_t va = __shfl_sync(0xffffffffu, a, k & 31), vb = __shfl_sync(0xffffffffu, b, k & 31);
    return k < c32 + 32 ? va : vb;
  }
  __device__ __forceinline__ void advance(int k, int lane) {
    if (k >= c32 + 32) {
      c32 += 32;
      a = b;
      b = boff[min(c32 + 32 + lane, last)];
    }
  }
};

template <typename T>
__device__ __forceinline__ void ld_quad(const T *p, T (&o)[4]);
template <>
__device__ __forceinline__ void ld_quad<float>(const float *p, float (&o)[4]) {
  const float4 v = *reinterpret_cast<const float4 *>(p);
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
  o[3] = v.w;
}
template <>
__device__ __forceinline__ void ld_quad<double>(const double *p, double (&o)[4]) {
  const double2 u = reinterpret_cast<const double2 *>(p)[0], w = reinterpret_cast<const double2 *>(p)[1];
  o[0] = u.x;
  o[1] = u.y;
  o[2] = w.x;
  o[3] = w.y;
}

// Row `lane` of a packed inverse into registers (zero outside the triangle).
template <typename VT, bool UPPER>
__device__ __forceinline__ void load_tinv_row(const VT *tinv, int lane, VT (&m)[BS]) {
  const int lo = tq_lo(lane, UPPER), hi = tq_hi(lane, UPPER), off = tq_off(lane, UPPER);
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    VT v[4] = {VT(0), VT(0), VT(0), VT(0)};
    if (q >= lo && q <= hi) ld_quad(tinv + 4 * (off + q - lo), v);
#pragma unroll
    for (int j = 0; j < 4; ++j) m[4 * q + j] = v[j];
  }
}

// sum_c m[c] t[c] with t read from shared memory as eight broadcast quads
// A 32-term dot product in N independent FMA chains (term c in chain c mod
// N), combined pairwise ((c0 + c1) + (c2 + c3)).  Eight chains for FP64
// measured slower than four (more registers, no shorter step).
template <typename VT>
struct FmaChains {
  static constexpr int N = 4;
  VT a[N];
  __device__ __forceinline__ FmaChains() {
#pragma unroll
    for (int i = 0; i < N; ++i) a[i] = VT(0);
  }
  __device__ __forceinline__ void add(int c, VT x, VT y) { a[c % N] = fma(x, y, a[c % N]); }
  __device__ __forceinline__ VT sum() {
#pragma unroll
    for (int st = 1; st < N; st *= 2)
#pragma unroll
      for (int i = 0; i + st < N; i += 2 * st) a[i] += a[i + st];
    return a[0];
  }
};

template <typename VT>
__device__ __forceinline__ VT apply_row(const VT (&m)[BS], const VT *tb) {
  FmaChains<VT> ch;
#pragma unroll
  for (int q = 0; q < 8; ++q) {
    VT t[4];
    ld_quad(tb + 4 * q, t);
#pragma unroll
    for (int u = 0; u < 4; ++u) ch.add(4 * q + u, m[4 * q + u], t[u]);
  }
  return ch.sum();
}

// Sparse dot products of one lane's row, eight entries at a time: the
// column and value loads of a batch are issued together, then the gathers of
// the solved values, then the FMAs (a dependent load-gather-FMA chain per
// entry would cost a shared-memory round trip each).

// slot-major entries: entry j of the lane's row at j * 32 + lane; columns
// relative to `base`
template <typename VT>
__device__ __forceinline__ VT slot_dot(const unsigned char *col, const VT *val, const VT *x, uint32_t base,
                                       uint32_t cnt, int lane) {
  VT a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  for (uint32_t j0 = 0; j0 < cnt; j0 += 8) {
    uint32_t c[8];
    VT v[8], g[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool ok = j0 + u < cnt;
      c[u] = ok ? (uint32_t)col[(j0 + u) * BS + lane] : 0u;
      v[u] = ok ? val[(j0 + u) * BS + lane] : VT(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) g[u] = x[base + c[u]];
#pragma unroll
    for (int u = 0; u < 8; u += 4) {
      a0 = fma(v[u], g[u], a0);
      a1 = fma(v[u + 1], g[u + 1], a1);
      a2 = fma(v[u + 2], g[u + 2], a2);
      a3 = fma(v[u + 3], g[u + 3], a3);
    }
  }
  return (a0 + a1) + (a2 + a3);
}

// contiguous entries [e0, e1) with piece-local columns, solved values at x[col & wmask]
template <typename VT, typename CT>
__device__ __forceinline__ VT run_dot(const CT *col, const VT *val, const VT *x, uint32_t wmask, uint32_t e0,
                                      uint32_t e1) {
  VT a0 = 0, a1 = 0, a2 = 0, a3 = 0;
  for (uint32_t e = e0; e < e1; e += 8) {
    uint32_t c[8];
    VT v[8], g[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const bool ok = e + u < e1;
      c[u] = ok ? (uint32_t)col[e + u] : 0u;
      v[u] = ok ? val[e + u] : VT(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) g[u] = x[c[u] & wmask];
#pragma unroll
    for (int u = 0; u < 8; u += 4) {
      a0 = fma(v[u], g[u], a0);
      a1 = fma(v[u + 1], g[u + 1], a1);
      a2 = fma(v[u + 2], g[u + 2], a2);
      a3 = fma(v[u + 3], g[u + 3], a3);
    }
  }
  return (a0 + a1) + (a2 + a3);
}

// sum of p[c0 .. c1)
template <typename VT>
__device__ __forceinline__ VT range_sum(const VT *p, uint32_t c0, uint32_t c1) {
  VT a0 = 0, a1 = 0;
  for (uint32_t c = c0; c < c1; c += 8) {
    VT v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) v[u] = c + u < c1 ? p[c + u] : VT(0);
#pragma unroll
    for (int u = 0; u < 8; u += 2) {
      a0 += v[u];
      a1 += v[u + 1];
    }
  }
  return a0 + a1;
}

// chunk g of `nchunk` interleaved chunks of `clen` entries (entry j at j * nchunk + g)
template <typename VT, typename CT>
__device__ __forceinline__ VT chunk_dot(const CT *col, const VT *val, const VT *x, uint32_t g, uint32_t nchunk,
                                        uint32_t clen) {
  VT a0 = 0, a1 = 0;
  for (uint32_t j0 = 0; j0 < clen; j0 += 4) {
    uint32_t c[4];
    VT v[4], xv[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      const bool ok = j0 + u < clen;
      const uint32_t at = (j0 + u) * nchunk + g;
      c[u] = ok ? (uint32_t)col[at] : 0u;
      v[u] = ok ? val[at] : VT(0);
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) xv[u] = x[c[u]];
    a0 = fma(v[0], xv[0], a0);
    a1 = fma(v[1], xv[1], a1);
    a0 = fma(v[2], xv[2], a0);
    a1 = fma(v[3], xv[3], a1);
  }
  return a0 + a1;
}

template <typename VT, typename InT>
__device__ __forceinline__ VT rhs_at(const VT *acc, const InT *in, int64_t i) {
  return acc ? __ldg(acc + i) : (VT)__ldg(in + i);
}

// Position of a record in a ring of mbarrier-guarded slots: record k sits in
// slot k mod R and completes phase k / R of that slot's barrier; each role
// walks its records in order, so the position advances by one per record.
struct RingPos {
  int slot = 0;
  uint32_t par = 0;
  __device__ __forceinline__ void next(int R) {
    if (++slot == R) {
      slot = 0;
      par ^= 1u;
    }
  }
};

// Block-wide barrier 0 over `n` threads, usable from the different loops of
// warp-specialised code (each thread of the block arrives once per use).
// Barrier 0 over n threads, returning the OR of every thread's `p`.
__device__ __forceinline__ bool cta_barrier_or(unsigned n, bool p) {
  uint32_t r;
  asm volatile(
      "{\n .reg .pred a, b;\n setp.ne.u32 a, %1, 0;\n bar.red.or.pred b, 0, %2, a;\n selp.u32 %0, 1, 0, b;\n}\n"
      : "=r"(r)
      : "r"((uint32_t)p), "r"(n)
      : "memory");
  return r != 0;
}

template <int SZ>
__device__ __forceinline__ void cp_async_small(void *smem, const void *gmem) {
  const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], %2;\n" ::"r"(s), "l"(gmem), "n"(SZ) : "memory");
}

template <typename VT>
struct W2Args {
  const NodeDesc *nodes;
  int node0, node1;   // pieces of this stage
  int wpb;            // warps (pieces) per thread block
  int nbuf;           // record slots per warp
  int bufbytes;       // bytes of a slot (16-aligned)
  int per_warp;       // shared-memory bytes per warp (16-aligned)
  int pf;             // records prefetched into L2 ahead of use (0: none)
  uint32_t wmask;     // window rows - 1 (a power of two)
  const unsigned char *blocks;
  const int64_t *blk_off;
  const VT *acc;      // rhs minus external sums, or null: the stage reads `in`
};

constexpr int kW2RhsRing = 4;  // warp format: blocks of right-hand side in flight per warp (a power of two)

// Shared memory of one warp of w2_kernel.
template <typename VT>
__host__ __device__ inline size_t w2_warp_bytes(int nbuf, size_t bufbytes, size_t window) {
  return al16(al16(8 * (size_t)nbuf) + BS * sizeof(VT) + (size_t)kW2RhsRing * BS * 8 + (size_t)nbuf * bufbytes +
              window * sizeof(VT));
}

// One warp per piece; per-warp shared memory: mbarriers, the broadcast
// buffer of t, the right-hand-side ring, the record ring, the window of
// solved values.  The right-hand side of block k+3 streams in with per-lane
// cp.async while block k is solved, so no register waits on a global load.
template <typename VT, typename InT, typename OutT, bool UPPER>
__global__ void __launch_bounds__(256) w2_kernel(W2Args<VT> a, const InT *__restrict__ in, OutT *__restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int piece = a.node0 + blockIdx.x * a.wpb + w;
  if (piece >= a.node1) return;  // the whole warp; no block-wide barrier follows
  const NodeDesc nd = a.nodes[piece];
  const int nb = nd.nblocks, NB = a.nbuf;
  unsigned char *base = smem + (size_t)w * a.per_warp;
  uint64_t *bar = reinterpret_cast<uint64_t *>(base);
  VT *tsh = reinterpret_cast<VT *>(base + al16(8 * (size_t)NB));
  double *rq = reinterpret_cast<double *>(tsh + BS);  // [kW2RhsRing][32] raw right-hand sides, 8-byte slots
  unsigned char *ring = reinterpret_cast<unsigned char *>(rq + kW2RhsRing * BS);
  VT *xw = reinterpret_cast<VT *>(ring + (size_t)NB * a.bufbytes);
  const uint32_t wmask = a.wmask;
  OffCache oc;
  oc.init(a.blk_off + nd.blk0, nb, lane);
  if (lane == 0) {
    for (int i = 0; i < NB; ++i) mbar_init(bar + i, 1);
    fence_mbar_init();
  }
  // padding entries (value 0) read the window at column 0: it starts at zero
  // so that they add 0, never 0 times stale shared memory
  for (uint32_t i = lane; i <= wmask; i += 32) xw[i] = VT(0);
  __syncwarp();
  auto issue = [&](int k, int slot) {  // all lanes (offset shuffles); lane 0 copies record k
    const int64_t o0 = oc.get(k), o1 = oc.get(k + 1);
    if (lane == 0) bulk_load(ring + (size_t)slot * a.bufbytes, a.blocks + o0, (uint32_t)(o1 - o0), bar + slot);
  };
  for (int k = 0; k < NB && k < nb; ++k) issue(k, k);
  auto fetch_rhs = [&](int k) {  // row `lane` of block k into its ring slot; one commit group per block
    if (k < nb) {
      const int row = (UPPER ? nb - 1 - k : k) * BS + lane;
      if (row < nd.rows) {
        void *dst = rq + (k & (kW2RhsRing - 1)) * BS + lane;
        if (a.acc) {
          if (sizeof(VT) == 8) cp_async_small<8>(dst, a.acc + nd.begin + row);
          else cp_async_small<4>(dst, a.acc + nd.begin + row);
        } else {
          if (sizeof(InT) == 8) cp_async_small<8>(dst, in + nd.begin + row);
          else cp_async_small<4>(dst, in + nd.begin + row);
        }
      }
    }
    cp_async_commit();
  };
  for (int k = 0; k < kW2RhsRing - 1; ++k) fetch_rhs(k);
  RingPos pos;
  int k = 0;
  bool ok = true;
  for (; k < nb; ++k) {
    fetch_rhs(k + kW2RhsRing - 1);
    ok = __all_sync(0xffffffffu, mbar_wait(bar + pos.slot, pos.par));
    if (!ok) break;
    cp_async_wait<kW2RhsRing - 1>();  // block k's right-hand side (this lane's own copy) is in
    const unsigned char *p = ring + (size_t)pos.slot * a.bufbytes;
    const uint4 h = *reinterpret_cast<const uint4 *>(p);
    const uint32_t nr = h.x, row0 = h.y, nent = h.z, csz = h.w;
    const W2Layout L = w2_layout(nent, csz, sizeof(VT));
    VT m[BS];
    load_tinv_row<VT, UPPER>(reinterpret_cast<const VT *>(p + L.o_tinv), lane, m);
    const uint16_t *eoff = reinterpret_cast<const uint16_t *>(p + L.o_eoff);
    const VT *val = reinterpret_cast<const VT *>(p + L.o_val);
    const uint32_t e0 = eoff[lane], e1 = eoff[lane + 1];
    const VT sum = csz == 2 ? run_dot(reinterpret_cast<const uint16_t *>(p + L.o_col), val, xw, wmask, e0, e1)
                            : run_dot(reinterpret_cast<const uint32_t *>(p + L.o_col), val, xw, wmask, e0, e1);
    const void *rp = rq + (k & (kW2RhsRing - 1)) * BS + lane;
    const VT q0 = a.acc ? *reinterpret_cast<const VT *>(rp) : (VT) * reinterpret_cast<const InT *>(rp);
    tsh[lane] = lane < (int)nr ? q0 - sum : VT(0);
    __syncwarp();
    const VT x = apply_row(m, tsh);
    if (lane < (int)nr) {
      xw[(row0 + lane) & wmask] = x;
      out[nd.begin + row0 + lane] = (OutT)x;
    }
    __syncwarp();  // slot and tsh free again
    oc.advance(k + NB, lane);  // the lowest record index used below
    if (k + NB < nb) {
      if (lane == 0) fence_proxy_async();
      issue(k + NB, pos.slot);
    }
    if (a.pf && k + a.pf < nb) {
      const int64_t o0 = oc.get(k + a.pf), o1 = oc.get(k + a.pf + 1);
      if (lane == 0) prefetch_l2(a.blocks + o0, (uint32_t)(o1 - o0));
    }
    pos.next(NB);
  }
  if (!ok) {  // give up: wait (bounded) for the copies still in flight, one per slot
    if (lane == 0) {
      atomicOr(&g_solve_status, 1u);
      RingPos q = pos;
      for (int j = k; j < nb && j < k + NB; ++j, q.next(NB)) (void)mbar_wait(bar + q.slot, q.par);
    }
    __syncwarp();
  }
  cp_async_wait<0>();
}

template <typename VT>
struct PipeArgs {
  const NodeDesc *nodes;
  int node0;         // piece = node0 + blockIdx.x
  int smem;          // dynamic shared memory of the launch (bytes)
  int ring;          // most ring slots (5..8): records k+1..k+3 in use, k+4 waited for, the rest in flight
  int maxchunk;      // most chunks of one block (chunk-sum buffer)
  int pf;            // records prefetched into L2 ahead of use
  const unsigned char *blocks;
  const int64_t *blk_off;
  const VT *acc;     // rhs minus external sums, or null: the stage reads `in`
};

// FP64 teams have at most 12 warps (170 registers a thread)
template <typename VT>
__host__ __device__ constexpr int pipe_max_threads() {
  return sizeof(VT) == 8 ? 384 : 512;
}

// Shared memory of pipe_kernel besides the record ring: the mbarriers (room
// for 8), then the reducer's broadcast buffer t[32], w[2][32], y[2][32], the
// chunk sums [2][maxchunk], and after the ring the piece's vector padded to
// whole blocks.
__host__ __device__ inline size_t pipe_vec_bytes_v(size_t vsz, int maxchunk) {
  return al16(vsz * (5 * BS + 2 * (size_t)maxchunk));
}
template <typename VT>
__host__ __device__ inline size_t pipe_vec_bytes(int maxchunk) {
  return pipe_vec_bytes_v(sizeof(VT), maxchunk);
}
// a pipeline piece's shared memory with a ring of `ring` slots
inline size_t pipe_piece_smem(size_t vsz, int maxchunk, int rows, int maxrec, int ring) {
  return al16(8 * 8) + pipe_vec_bytes_v(vsz, maxchunk) + (size_t)((rows + BS - 1) / BS * BS) * vsz +
         (size_t)ring * al16((size_t)maxrec);
}
// a k-team piece's shared memory with a ring of `ring` records
inline size_t team_piece_smem(size_t vsz, int rows, int maxrec, int ring) {
  return (size_t)ring * al16((size_t)maxrec) + 2 * (size_t)BS * KW * vsz + (size_t)rows * KW * vsz;
}

// One thread block per piece.  In step s:
//   warp 0 (solver)   x_s = w_s + y_s - P_s x_{s-1}, with P_s's row and the
//                     broadcast x_{s-1} in registers; then reads x_s back as
//                     eight broadcast quads and P_{s+1}'s row;
//   warp 1 (reducer)  w_{s+1} = T^-1 (acc - chunk sums) of block s+1, then
//                     the inverse row of block s+2;
//   warp 2 (mixer)    y_{s+1} = -Q_{s+1} x_{s-1}, then Q's row of block s+2;
//   warp 3 (streamer) copies record s+RING into the slot of record s and,
//                     one thread, waits for record s+4 (the next barrier then
//                     publishes it to every warp);
//   warps 4..         far chunk sums of block s+2.
// One block-wide barrier per step (bar.red.or, carrying the streamer's
// failure flag).  The piece's right-hand side, then its solution, live in
// shared memory (xs).
template <typename VT, typename InT, typename OutT, bool UPPER>
__global__ void __launch_bounds__(pipe_max_threads<VT>(), 1) pipe_kernel(PipeArgs<VT> a, const InT *__restrict__ in,
                                                                         OutT *__restrict__ out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const NodeDesc nd = a.nodes[a.node0 + blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int nb = nd.nblocks;
  const int stride = pq_stride(sizeof(VT));
  // this piece's ring: slots of its longest record, as many (up to a.ring)
  // as the launch's shared memory holds besides the vectors and its rows
  const int rows_pad = (nd.rows + BS - 1) / BS * BS;
  const size_t slot_bytes = al16((size_t)nd.maxrec);
  const size_t head = al16(8 * 8) + pipe_vec_bytes<VT>(a.maxchunk) + (size_t)rows_pad * sizeof(VT);
  const int RING = min(a.ring, (int)(((size_t)a.smem - min((size_t)a.smem, head)) / slot_bytes));
  if (RING < kPipeRingMin) {  // excluded by the plan (every piece fits the smallest ring)
    if (tid == 0) atomicOr(&g_solve_status, 2u);
    return;
  }
  uint64_t *bar = reinterpret_cast<uint64_t *>(smem);
  VT *tb = reinterpret_cast<VT *>(smem + al16(8 * 8));
  VT *wbuf = tb + BS;        // [2][32]
  VT *ybuf = wbuf + 2 * BS;  // [2][32]
  VT *part = ybuf + 2 * BS;  // [2][maxchunk]
  unsigned char *ring = reinterpret_cast<unsigned char *>(tb) + pipe_vec_bytes<VT>(a.maxchunk);
  VT *xs = reinterpret_cast<VT *>(ring + (size_t)RING * slot_bytes);
  OffCache oc;
  if (warp == 3) oc.init(a.blk_off + nd.blk0, nb, lane);
  if (tid == 0) {
    for (int i = 0; i < RING; ++i) mbar_init(bar + i, 1);
    fence_mbar_init();
  }
  // the piece's right-hand side into shared memory (zeros past its rows),
  // eight loads in flight per thread
  for (int r0 = tid; r0 < rows_pad; r0 += 8 * (int)blockDim.x) {
    VT v[8];
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int r = r0 + u * (int)blockDim.x;
      v[u] = r < nd.rows ? rhs_at(a.acc, in, nd.begin + r) : VT(0);
    }
#pragma unroll
    for (int u = 0; u < 8; ++u) {
      const int r = r0 + u * (int)blockDim.x;
      if (r < rows_pad) xs[r] = v[u];
    }
  }
  __syncthreads();
  auto slot_ptr = [&](int slot) { return ring + (size_t)slot * slot_bytes; };
  // warp 3 streams the records: into every slot first, then record k into
  // the slot of record k - RING (all reads of that slot finished before the
  // last barrier); its lane 0 waits for record k four steps before use, so
  // that after the next barrier every warp may read records up to k (each
  // role loads its next step's operands a step ahead).
  RingPos ld, wt;
  int issued = 0, waited = 0;
  bool failed = false;  // warp 3 lane 0: a bounded wait gave up
  auto issue = [&](int k) {
    const int64_t o0 = oc.get(k), o1 = oc.get(k + 1);
    if (lane == 0) bulk_load(slot_ptr(ld.slot), a.blocks + o0, (uint32_t)(o1 - o0), bar + ld.slot);
    ld.next(RING);
    issued = k + 1;
  };
  auto wait_next = [&]() {  // warp 3 lane 0: the next record in order
    if (!mbar_wait(bar + wt.slot, wt.par)) {
      atomicOr(&g_solve_status, 1u);
      failed = true;
    }
    wt.next(RING);
    ++waited;
  };
  if (warp == 3) {
    for (int k = 0; k < RING && k < nb; ++k) issue(k);
    if (lane == 0)
      while (waited < 4 && waited < nb && !failed) wait_next();
  }
  bool stop = __syncthreads_or(failed);
  // Each role runs its own loop over the steps (registers are then allocated
  // per role); every loop passes the same block-wide barrier once per step,
  // which also ORs the streamer's failure flag into `stop` (uniform across
  // the block, without a shared-memory read on any role's chain).
  const unsigned nthreads = blockDim.x;
  if (warp == 0) {  // solver: x_s = w_s + y_s - P_s x_{s-1}
    VT pr[BS], xb[BS];
#pragma unroll
    for (int c = 0; c < BS; ++c) xb[c] = VT(0);
    uint32_t s_nr = 0, s_row0 = 0;
    RingPos rp;  // record of the solver's next block
    for (int s = -2; s < nb; ++s) {
      if (!stop) {
        if (s >= 0) {
          FmaChains<VT> ch;
#pragma unroll
          for (int c = 0; c < BS; ++c) ch.add(c, pr[c], xb[c]);
          const VT x = (wbuf[(s & 1) * BS + lane] + ybuf[(s & 1) * BS + lane]) - ch.sum();
          if (lane < (int)s_nr) {
            xs[s_row0 + lane] = x;
            out[nd.begin + s_row0 + lane] = (OutT)x;
          }
          __syncwarp();
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            VT t[4];
            ld_quad(xs + s_row0 + 4 * q, t);
#pragma unroll
            for (int u = 0; u < 4; ++u) xb[4 * q + u] = t[u];
          }
        }
        if (s + 1 >= 0 && s + 1 < nb) {  // block s+1: header and P's row
          const unsigned char *p = slot_ptr(rp.slot);
          rp.next(RING);
          const uint4 h0 = *reinterpret_cast<const uint4 *>(p);
          s_nr = h0.x;
          s_row0 = h0.y;
          const VT *P = reinterpret_cast<const VT *>(p + 64 + sizeof(VT) * 4 * TQ) + lane * stride;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            VT t[4];
            ld_quad(P + 4 * q, t);
#pragma unroll
            for (int u = 0; u < 4; ++u) pr[4 * q + u] = t[u];
          }
        }
      }
      stop = cta_barrier_or(nthreads, failed);
    }
  } else if (warp == 1) {  // reducer: w of block s+1 = T^-1 (acc - chunk sums)
    VT m[BS];                // inverse row of block s+1, loaded in step s-1
    uint32_t r_nr = 0, r_row0 = 0, c0 = 0, c1 = 0;
    RingPos rp;
    auto load_next = [&](VT (&mm)[BS], uint32_t &nr, uint32_t &row0, uint32_t &a0, uint32_t &a1) {
      const unsigned char *p = slot_ptr(rp.slot);
      rp.next(RING);
      load_tinv_row<VT, UPPER>(reinterpret_cast<const VT *>(p + 64), lane, mm);
      const uint4 h0 = *reinterpret_cast<const uint4 *>(p);
      const uint16_t *crow = reinterpret_cast<const uint16_t *>(p + pipe_o_crow(sizeof(VT)));
      nr = h0.x;
      row0 = h0.y;
      a0 = crow[lane];
      a1 = crow[lane + 1];
    };
    if (nb > 0) load_next(m, r_nr, r_row0, c0, c1);  // block 0 (records 0..3 are in)
    for (int s = -2; s < nb; ++s) {
      const int bk = s + 1;
      if (!stop && bk >= 0 && bk < nb) {
        // this step's reads first: shared-memory requests are served in
        // order, so the next block's operands are loaded after them
        const VT far = range_sum(part + (size_t)(bk & 1) * a.maxchunk, c0, c1);
        tb[lane] = lane < (int)r_nr ? xs[r_row0 + lane] - far : VT(0);
        __syncwarp();
        wbuf[(bk & 1) * BS + lane] = apply_row(m, tb);
        if (bk + 1 < nb) load_next(m, r_nr, r_row0, c0, c1);
      }
      stop = cta_barrier_or(nthreads, failed);
    }
  } else if (warp == 2) {  // mixer: y of block s+1 = -Q x of block s-1
    VT qr[BS];               // Q's row of block s+1, loaded in step s-1
    uint32_t m_pprow0 = 0;
    RingPos rp;
    auto load_next = [&](VT (&qq)[BS], uint32_t &pprow0) {
      const unsigned char *p = slot_ptr(rp.slot);
      rp.next(RING);
      pprow0 = reinterpret_cast<const uint32_t *>(p)[3];
      const VT *Q = reinterpret_cast<const VT *>(p + 64 + sizeof(VT) * (4 * TQ + (size_t)BS * stride)) + lane * stride;
#pragma unroll
      for (int q = 0; q < 8; ++q) {
        VT t[4];
        ld_quad(Q + 4 * q, t);
#pragma unroll
        for (int u = 0; u < 4; ++u) qq[4 * q + u] = t[u];
      }
    };
    if (nb > 0) load_next(qr, m_pprow0);
    for (int s = -2; s < nb; ++s) {
      const int bk = s + 1;
      if (!stop && bk >= 0 && bk < nb) {
        VT y = VT(0);
        if (bk >= 2) {
          FmaChains<VT> ch;
#pragma unroll
          for (int q = 0; q < 8; ++q) {
            VT xx[4];
            ld_quad(xs + m_pprow0 + 4 * q, xx);
#pragma unroll
            for (int u = 0; u < 4; ++u) ch.add(4 * q + u, qr[4 * q + u], xx[u]);
          }
          y = -ch.sum();
        }
        ybuf[(bk & 1) * BS + lane] = y;
        if (bk + 1 < nb) load_next(qr, m_pprow0);  // after this step's reads (served in order)
      }
      stop = cta_barrier_or(nthreads, failed);
    }
  } else if (warp == 3) {  // streams the records
    for (int s = -2; s < nb; ++s) {
      if (!stop && s >= 0) {  // record s+RING into the slot of record s (free since the last barrier)
        const int k = s + RING;
        oc.advance(a.pf ? min(k, s + a.pf) : k, lane);  // the lowest record index used this step
        if (k < nb) issue(k);
        if (a.pf && s + a.pf < nb) {
          const int64_t o0 = oc.get(s + a.pf), o1 = oc.get(s + a.pf + 1);
          if (lane == 0) prefetch_l2(a.blocks + o0, (uint32_t)(o1 - o0));
        }
        if (lane == 0 && s + 4 < nb) wait_next();  // record s+4, read from the next step on
      }
      stop = cta_barrier_or(nthreads, failed);
    }
  } else {  // gatherers: far sums of block s+2
    const int g = tid - 32 * kPipeRoleWarps;
    RingPos rp;
    rp.next(RING);
    rp.next(RING);  // record 2: the gatherers' first block in step 0 (blocks 0, 1 have no far entries)
    // chunk g of the next block: its first kPipeGPre entries' columns and values
    constexpr int GP = 4;
    uint32_t gcol[GP] = {0, 0, 0, 0}, nchunk = 0, clen = 0, csz = 2, o_fc = 0, o_fv = 0;
    VT gval[GP] = {VT(0), VT(0), VT(0), VT(0)};
    const unsigned char *gp = nullptr;
    auto load_next = [&](int bk) {  // block bk's header and this thread's first entries
      gp = slot_ptr(rp.slot);
      rp.next(RING);
      const uint4 h1 = *reinterpret_cast<const uint4 *>(gp + 16);
      const uint4 h2 = *reinterpret_cast<const uint4 *>(gp + 32);
      nchunk = h1.x;
      clen = h1.y;
      csz = h1.z;
      o_fc = h2.x;
      o_fv = h2.y;
      (void)bk;
#pragma unroll
      for (int u = 0; u < GP; ++u) {
        const bool ok = g < (int)nchunk && (uint32_t)u < clen;
        const uint32_t at = (uint32_t)u * nchunk + (uint32_t)g;
        gcol[u] = !ok ? 0u
                      : csz == 2 ? (uint32_t)reinterpret_cast<const uint16_t *>(gp + o_fc)[at]
                                 : reinterpret_cast<const uint32_t *>(gp + o_fc)[at];
        gval[u] = ok ? reinterpret_cast<const VT *>(gp + o_fv)[at] : VT(0);
      }
    };
    if (nb > 2) load_next(2);
    for (int s = -2; s < nb; ++s) {
      if (!stop) {
        const int bk = s + 2;
        if (bk >= 2 && bk < nb) {
          // this step: the preloaded entries of block bk, the rest from the record
          if (g < (int)nchunk) {
            VT xg[GP];
#pragma unroll
            for (int u = 0; u < GP; ++u) xg[u] = xs[gcol[u]];
            VT a0 = 0, a1 = 0;
#pragma unroll
            for (int u = 0; u < GP; u += 2) {
              a0 = fma(gval[u], xg[u], a0);
              a1 = fma(gval[u + 1], xg[u + 1], a1);
            }
            VT sum = a0 + a1;
            if (clen > (uint32_t)GP) {
              const uint32_t base = (uint32_t)GP * nchunk + (uint32_t)g;
              const VT *fv = reinterpret_cast<const VT *>(gp + o_fv) + (uint32_t)GP * nchunk;
              sum += csz == 2 ? chunk_dot(reinterpret_cast<const uint16_t *>(gp + o_fc) + (uint32_t)GP * nchunk, fv, xs,
                                          (uint32_t)g, nchunk, clen - GP)
                              : chunk_dot(reinterpret_cast<const uint32_t *>(gp + o_fc) + (uint32_t)GP * nchunk, fv, xs,
                                          (uint32_t)g, nchunk, clen - GP);
              (void)base;
            }
            part[(size_t)(bk & 1) * a.maxchunk + g] = sum;
          }
          if (bk + 1 < nb) load_next(bk + 1);
        }
      }
      stop = cta_barrier_or(nthreads, failed);
    }
  }
  if (stop && warp == 3 && lane == 0) {
    // copies that may still be in flight: those issued and not waited for (one per slot)
    while (waited < issued) {
      (void)mbar_wait(bar + wt.slot, wt.par);
      wt.next(RING);
      ++waited;
    }
  }
}

}  // namespace

// ---- plan construction ---------------------------------------------------------------

// SM count of the current device (a scheduling heuristic only: without a
// device, as in host-side plan checks, the GB300's 152 is assumed).
static int sm_count() {
  int dev = 0, c = 0;
  if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess &&
      c > 0)
    return c;
  (void)cudaGetLastError();
  return 152;
}

// Host copy of one direction's stream (tests/stream_emulator.cu executes it on the CPU).
struct HostStreamCopy {
  std::vector<unsigned char> blocks;
  std::vector<int64_t> blk_off;
  std::vector<NodeDesc> desc;
  std::vector<int64_t> ext_rp;
  std::vector<int32_t> ext_ci;
  std::vector<double> ext_v;
  std::vector<int> stage_ptr;
  std::vector<int> stage_fmt;
  std::vector<int> stage_window;
};

constexpr size_t kSmemCap = 220 * 1024;      // dynamic shared memory a launch may use
constexpr int kW2Ring = 4;                   // warp format: record slots per warp
constexpr int kW2WindowMax = 8192;           // warp format: most rows in a window
constexpr size_t kW2WarpBudget = 56 * 1024;  // warp format: shared memory of one warp (at least 4 warps per SM)

// Pipeline team size of a stage with `pieces` pieces: 16 warps where at
// most one piece runs per SM, fewer (several teams per SM) beyond.
static int pipe_warps_for(int pieces, int sms, size_t vsz) {
  return pieces <= sms ? (vsz == 8 ? 12 : 16) : pieces <= 2 * sms ? 8 : 6;
}

static void build_dir_streams(const std::vector<int64_t> &rp, const std::vector<int32_t> &ci,
                              const std::vector<double> &v, int64_t n, const std::vector<TreeNode> &tnodes,
                              bool upper, bool fp32, int fmt_mode, int kwidth, StreamDir &D, cudaStream_t s,
                              HostStreamCopy *host_copy = nullptr) {
  const size_t vsz = fp32 ? 4 : 8;
  const int sms = sm_count();
  int maxdepth = 1;
  for (auto &nd : tnodes) maxdepth = std::max(maxdepth, nd.depth);
  struct Piece {
    int64_t b, e;
    int fmt;     // FMT_WARP, FMT_PIPE or FMT_KTEAM
    int warps;   // pipeline / k-team: warps of the team
    int window;  // warp format: window rows
  };
  // Pieces grow in processing order (ascending blocks forward, descending
  // backward).  The record of the block at processing position q of a piece
  // that starts at position p holds its rows' entries whose columns lie in
  // positions p..q-1 of the node (entries in earlier pieces are external);
  // rec_bound is an upper bound of its length in the given format (the exact
  // length for the pipeline format, split by distance 1, 2, more), with
  // `gth` gatherer or helper threads.
  struct NodeView {
    int64_t b, e, nb;
  };
  auto rec_bound = [&](const NodeView &v, int fmt, int gth, int64_t q, int64_t p) -> size_t {
    const int64_t bq = upper ? v.nb - 1 - q : q;
    const int64_t r0 = v.b + bq * BS, r1 = std::min(v.e, r0 + BS);
    const size_t csz = v.e - v.b > 65535 ? 4 : 2;
    size_t cnt = 0, far = 0;
    uint32_t rf[BS] = {};
    for (int64_t i = r0; i < r1; ++i) {
      for (int64_t t = rp[i]; t < rp[i + 1]; ++t) {
        const int64_t c = ci[t];
        if (c < v.b || c >= v.e || (c >= r0 && c < r1)) continue;
        const int64_t cb = (c - v.b) / BS;
        const int64_t d = upper ? cb - bq : bq - cb;  // blocks back in processing order
        if (d > q - p) continue;                      // in an earlier piece: external
        ++cnt;
        if (d > 2) {
          ++far;
          ++rf[i - r0];
        }
      }
    }
    if (fmt == FMT_WARP) return w2_record_bound(cnt, vsz, csz);
    if (fmt == FMT_PIPE) return pipe_record_len(rf, (uint32_t)far, gth, vsz, csz);
    return team_record_bound(cnt, (size_t)gth, vsz, csz);
  };
  // Cuts a node into pieces of whole blocks whose shared memory fits:
  // fixed + nrec * (largest record) + rows * row_bytes <= cap and rows <=
  // max_rows.  Pieces come back in row order.  False if a single block does
  // not fit.
  auto cut = [&](const NodeView &v, int fmt, int gth, size_t fixed, size_t nrec, size_t row_bytes,
                 int64_t max_rows, size_t cap, std::vector<std::pair<int64_t, int64_t>> &out) {
    auto rows_of = [&](int64_t p, int64_t q) {  // rows of processing positions [p, q)
      return upper ? std::min(v.e, v.b + (v.nb - p) * BS) - (v.b + (v.nb - q) * BS)
                   : std::min(v.e, v.b + q * BS) - (v.b + p * BS);
    };
    int64_t p = 0;
    while (p < v.nb) {
      int64_t q = p;
      size_t mx = 0;
      while (q < v.nb) {
        const size_t m2 = std::max(mx, al16(rec_bound(v, fmt, gth, q, p)));
        const int64_t rows = rows_of(p, q + 1);
        if (q > p && (fixed + nrec * m2 + (size_t)rows * row_bytes > cap || rows > max_rows)) break;
        mx = m2;
        ++q;
      }
      if (fixed + nrec * mx + (size_t)rows_of(p, q) * row_bytes > cap) return false;
      if (upper) out.push_back({v.b + (v.nb - q) * BS, std::min(v.e, v.b + (v.nb - p) * BS)});
      else out.push_back({v.b + p * BS, std::min(v.e, v.b + q * BS)});
      p = q;
    }
    if (upper) std::reverse(out.begin(), out.end());
    return true;
  };
  // longest row-column distance inside [b, e)
  auto reach_of = [&](int64_t b, int64_t e) {
    int64_t r = 0;
    for (int64_t i = b; i < e; ++i)
      for (int64_t q = rp[i]; q < rp[i + 1]; ++q)
        if (ci[q] >= b && ci[q] < e) r = std::max<int64_t>(r, std::abs(i - (int64_t)ci[q]));
    return r;
  };
  auto pow2_at_least = [](int64_t x) {
    int64_t w = 64;
    while (w < x) w <<= 1;
    return w;
  };
  std::vector<Piece> pieces;
  D.stage_ptr.assign(1, 0);
  for (int st = 0; st < maxdepth; ++st) {
    const int depth = upper ? st + 1 : maxdepth - st;
    std::vector<std::pair<int64_t, int64_t>> nodes;
    for (auto &nd : tnodes)
      if (nd.depth == depth && std::min(nd.end, n) > nd.begin) nodes.push_back({nd.begin, std::min(nd.end, n)});
    if (nodes.empty()) continue;
    const int P = (int)nodes.size();
    int fmt = kwidth > 1 ? FMT_KTEAM : fmt_mode == 0 ? FMT_WARP : fmt_mode == 2 ? FMT_PIPE : P >= 2 * sms ? FMT_WARP : FMT_PIPE;
    std::vector<std::vector<Piece>> per_node(P);
    for (int attempt = 0; attempt < 2; ++attempt) {
      std::vector<char> node_ok(P, 1);
      parallel_for(P, [&](int64_t j0, int64_t j1) {
        for (int64_t j = j0; j < j1; ++j) {
          const NodeView v{nodes[j].first, nodes[j].second, (nodes[j].second - nodes[j].first + BS - 1) / BS};
          std::vector<std::pair<int64_t, int64_t>> rng;
          per_node[j].clear();
          bool ok;
          if (fmt == FMT_WARP) {
            const int64_t W = std::min<int64_t>(pow2_at_least(std::min<int64_t>(reach_of(v.b, v.e) + BS + 1, v.e - v.b)),
                                                kW2WindowMax);
            const size_t fixed = al16(8 * kW2Ring) + BS * vsz + (size_t)kW2RhsRing * BS * 8 + (size_t)W * vsz;
            // rows per piece bounded by the window: a piece of at most W rows
            // never reads outside it, whatever the node's reach
            ok = cut(v, fmt, 0, fixed, kW2Ring, 0, W >= kW2WindowMax ? W : INT64_MAX, kW2WarpBudget, rng);
            for (auto &r : rng) per_node[j].push_back(Piece{r.first, r.second, FMT_WARP, 1, (int)W});
          } else if (fmt == FMT_PIPE) {
            const int warps = pipe_warps_for(P, sms, vsz);
            const int gth = 32 * (warps - kPipeRoleWarps);
            const size_t fixed = al16(8 * 8) + al16(vsz * (5 * BS + 2 * (size_t)gth)) + BS * vsz;  // + block padding
            // the ring the pieces are cut for, the smallest one where a
            // single block's record would not fit a deeper one
            ok = cut(v, fmt, gth, fixed, kPipeRingCut, vsz, 1 << 30, kSmemCap, rng);
            if (!ok) {
              rng.clear();
              ok = cut(v, fmt, gth, fixed, kPipeRingMin, vsz, 1 << 30, kSmemCap, rng);
            }
            for (auto &r : rng) per_node[j].push_back(Piece{r.first, r.second, FMT_PIPE, warps, 0});
          } else {
            const int warps = 8, hth = 32 * (warps - 1);
            const size_t fixed = 2 * (size_t)BS * KW * vsz;
            ok = cut(v, fmt, hth, fixed, TEAM_RING, vsz * KW, 65535, kSmemCap, rng);
            for (auto &r : rng) per_node[j].push_back(Piece{r.first, r.second, FMT_KTEAM, warps, 0});
          }
          node_ok[j] = ok;
        }
      }, 1);
      int bad = -1;
      for (int j = 0; j < P && bad < 0; ++j)
        if (!node_ok[j]) bad = j;
      if (bad < 0) break;
      if (fmt != FMT_WARP)
        throw Error(RCHOL_ERR_INTERNAL, "a 32-row block of G is too dense for the shared-memory solve (depth " +
                                            std::to_string(depth) + ", node rows " + std::to_string(nodes[bad].first) +
                                            ".." + std::to_string(nodes[bad].second) + ")");
      fmt = FMT_PIPE;  // records too large for a warp's share: this depth in the pipeline format
    }
    std::vector<std::vector<Piece>> by_index;  // piece j of every node of this depth
    for (auto &ps : per_node) {
      if (upper) std::reverse(ps.begin(), ps.end());  // backward: last piece first
      if (by_index.size() < ps.size()) by_index.resize(ps.size());
      for (size_t j = 0; j < ps.size(); ++j) by_index[j].push_back(ps[j]);
    }
    for (auto &grp : by_index) {
      for (auto &pc : grp) pieces.push_back(pc);
      D.stage_ptr.push_back((int)pieces.size());
    }
  }
  const int np = (int)pieces.size();
  std::vector<int32_t> piece_of(n, -1);
  for (int k = 0; k < np; ++k)
    for (int64_t i = pieces[k].b; i < pieces[k].e; ++i) piece_of[i] = k;
  // external CSR (entries outside the row's piece, diagonal excluded)
  std::vector<int64_t> ext_rp(n + 1, 0);
  parallel_for(n, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) {
      const int k = piece_of[i];
      int64_t c = 0;
      for (int64_t q = rp[i]; q < rp[i + 1]; ++q) c += (ci[q] < pieces[k].b || ci[q] >= pieces[k].e);
      ext_rp[i + 1] = c;
    }
  }, 1 << 14);
  for (int64_t i = 0; i < n; ++i) ext_rp[i + 1] += ext_rp[i];
  const int64_t next = ext_rp[n];
  std::vector<int32_t> eci(next);
  std::vector<double> ev(next);
  parallel_for(n, [&](int64_t i0, int64_t i1) {
    for (int64_t i = i0; i < i1; ++i) {
      const int k = piece_of[i];
      int64_t w = ext_rp[i];
      for (int64_t q = rp[i]; q < rp[i + 1]; ++q)
        if (ci[q] < pieces[k].b || ci[q] >= pieces[k].e) {
          eci[w] = ci[q];
          ev[w] = v[q];
          ++w;
        }
    }
  }, 1 << 14);
  // block records, the largest pieces first (they take the longest)
  std::vector<PieceBuild> built(np);
  std::vector<int32_t> chunks(np, 0);
  std::vector<int> by_size(np);
  for (int k = 0; k < np; ++k) by_size[k] = k;
  std::stable_sort(by_size.begin(), by_size.end(),
                   [&](int x, int y) { return pieces[x].e - pieces[x].b > pieces[y].e - pieces[y].b; });
  parallel_for(np, [&](int64_t k0, int64_t k1) {
    for (int64_t kk = k0; kk < k1; ++kk) {
      const int k = by_size[kk];
      const Piece &pc = pieces[k];
      if (pc.fmt == FMT_WARP) {
        int64_t reach = 0;
        build_w2_piece(rp, ci, v, pc.b, pc.e, upper, vsz, built[k], reach);
        if (reach + BS >= pc.window && pc.window < pc.e - pc.b)
          throw Error(RCHOL_ERR_INTERNAL, "warp-format window shorter than the piece's reach");
      } else if (pc.fmt == FMT_PIPE) {
        build_pipe_piece(rp, ci, v, pc.b, pc.e, upper, vsz, 32 * (pc.warps - kPipeRoleWarps), built[k], chunks[k]);
      } else {
        build_team_piece(rp, ci, v, pc.b, pc.e, upper, vsz, 32 * (pc.warps - 1), true, built[k], chunks[k]);
      }
    }
  }, 1);
  std::vector<NodeDesc> desc(np);
  std::vector<int64_t> blk_off;
  int64_t total = 0;
  D.sparse_nnz = 0;
  for (int k = 0; k < np; ++k) {
    desc[k].begin = pieces[k].b;
    desc[k].rows = (int32_t)(pieces[k].e - pieces[k].b);
    desc[k].nblocks = (int32_t)(built[k].offs.size() - 1);
    desc[k].blk0 = (int64_t)blk_off.size();
    desc[k].maxrec = built[k].maxrec;
    desc[k].wide = desc[k].rows > 65535;
    desc[k].maxchunk = chunks[k];
    desc[k].pad_ = 0;
    for (int64_t o : built[k].offs) blk_off.push_back(total + o);
    total += (int64_t)built[k].bytes.size();
    D.sparse_nnz += built[k].sparse;
  }
  // every byte is written by one piece's copy: no zero fill
  std::unique_ptr<unsigned char[]> all(new unsigned char[std::max<int64_t>(total, 1)]);
  parallel_for(np, [&](int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; ++k)
      std::memcpy(all.get() + blk_off[desc[k].blk0], built[k].bytes.data(), built[k].bytes.size());
  }, 1);
  built.clear();
  // stages
  D.stage_rows.clear();
  D.stage_maxrec.clear();
  D.stage_fmt.clear();
  D.stage_warps.clear();
  D.stage_chunks.clear();
  D.stage_window.clear();
  D.stage_ext.clear();
  D.stage_ext_lanes.clear();
  D.stage_smem.clear();
  D.stage_row_ptr.assign(1, 0);
  D.steps = 0;
  std::vector<int32_t> srows;
  for (size_t st = 0; st + 1 < D.stage_ptr.size(); ++st) {
    int rows = 0, maxrec = 16, steps = 0, maxchunk = 0, window = 0;
    int64_t ext = 0, nrow = 0;
    for (int k = D.stage_ptr[st]; k < D.stage_ptr[st + 1]; ++k) {
      rows = std::max(rows, desc[k].rows);
      maxrec = std::max(maxrec, desc[k].maxrec);
      steps = std::max(steps, desc[k].nblocks);
      maxchunk = std::max(maxchunk, desc[k].maxchunk);
      window = std::max(window, pieces[k].window);
      for (int64_t i = desc[k].begin; i < desc[k].begin + desc[k].rows; ++i) srows.push_back((int32_t)i);
      ext += ext_rp[desc[k].begin + desc[k].rows] - ext_rp[desc[k].begin];
      nrow += desc[k].rows;
    }
    const Piece &p0 = pieces[D.stage_ptr[st]];
    const double avg = nrow ? (double)ext / (double)nrow : 0.0;
    // per ring depth, the launch's shared memory: the largest of its pieces'
    // (each capped where that piece's deeper ring no longer fits); every
    // piece must fit the smallest ring
    std::array<int, 9> sm{};
    if (p0.fmt != FMT_WARP) {
      const bool pipe = p0.fmt == FMT_PIPE;
      const int rmin = pipe ? kPipeRingMin : TEAM_RING_MIN, rmax = pipe ? kPipeRingMax : TEAM_RING_MAX;
      const int mc = std::max(1, maxchunk);
      for (int k = D.stage_ptr[st]; k < D.stage_ptr[st + 1]; ++k) {
        auto need = [&](int r) {
          return pipe ? pipe_piece_smem(vsz, mc, desc[k].rows, desc[k].maxrec, r)
                      : team_piece_smem(vsz, desc[k].rows, desc[k].maxrec, r);
        };
        if (need(rmin) > kSmemCap) throw Error(RCHOL_ERR_INTERNAL, "solve piece exceeds shared memory");
        for (int r = rmin; r <= rmax; ++r) sm[r] = std::max<int>(sm[r], (int)std::min(kSmemCap, need(r)));
      }
    }
    D.stage_smem.push_back(sm);
    D.stage_rows.push_back(rows);
    D.stage_maxrec.push_back(maxrec);
    D.stage_fmt.push_back(p0.fmt);
    D.stage_warps.push_back(p0.warps);
    D.stage_chunks.push_back(std::max(1, maxchunk));
    D.stage_window.push_back(window);
    D.stage_ext.push_back(ext > 0 ? 1 : 0);
    D.stage_ext_lanes.push_back(avg < 6 ? 1 : avg < 24 ? 4 : avg < 96 ? 8 : 32);
    D.stage_row_ptr.push_back((int64_t)srows.size());
    D.steps += steps;
  }
  D.nblocks = (int64_t)blk_off.size() - np;
  D.ext_nnz = next;
  if (host_copy) {
    host_copy->blocks.assign(all.get(), all.get() + total);
    host_copy->blk_off = blk_off;
    host_copy->desc = desc;
    host_copy->ext_rp = ext_rp;
    host_copy->ext_ci = eci;
    host_copy->ext_v = ev;
    host_copy->stage_ptr = D.stage_ptr;
    host_copy->stage_fmt = D.stage_fmt;
    host_copy->stage_window = D.stage_window;
    return;
  }
  D.blocks.upload(all.get(), (size_t)total, s);
  D.blk_off.upload(blk_off.data(), blk_off.size(), s);
  D.nodes.upload(desc.data(), np, s);
  D.ext_rp.upload(ext_rp.data(), n + 1, s);
  D.ext_ci.upload(eci.data(), next, s);
  if (!fp32) D.ext_v64.upload(ev.data(), next, s);
  std::vector<float> ev32;
  if (fp32) {
    ev32.resize(next);
    parallel_for(next, [&](int64_t q0, int64_t q1) {
      for (int64_t q = q0; q < q1; ++q) ev32[q] = (float)ev[q];
    }, 1 << 20);
    D.ext_v32.upload(ev32.data(), next, s);
  }
  D.srows.upload(srows.data(), srows.size(), s);
  RCHOL_CUDA(cudaStreamSynchronize(s));
}

// Builds both directions' streams for pieces holding `kwidth` values per row.
static void build_streams_width(const rchol_factor_s &F, int kwidth, StreamDir &fwd, StreamDir &bwd,
                                cudaStream_t s) {
  const int64_t n = F.n, nnz = F.nnz;
  const bool fp32 = F.precision == RCHOL_PREC_FP32;
#ifdef RCHOL_DEVICE_CHECKS
  RCHOL_CUDA(cudaMemcpyToSymbol(dbg_n, &n, sizeof(n)));
#endif
  std::vector<int64_t> rp(n + 1);
  std::vector<int32_t> ci(nnz);
  std::vector<double> v(nnz);
  F.lrp.download(rp.data(), n + 1, s);
  F.lci.download(ci.data(), nnz, s);
  F.lv.download(v.data(), nnz, s);
  RCHOL_CUDA(cudaStreamSynchronize(s));
  // Schedule knob (tuning only; every setting solves exactly the same
  // system): RCHOL_TRSV_FORMAT = 0 warp format everywhere, 1 by stage
  // (default: warp format where a depth has many nodes, pipeline format
  // at the top of the tree), 2 pipeline format everywhere.
  int fmt_mode = 1;
  if (const char *e = getenv("RCHOL_TRSV_FORMAT")) fmt_mode = std::max(0, std::min(2, atoi(e)));
  build_dir_streams(rp, ci, v, n, F.nodes, false, fp32, fmt_mode, kwidth, fwd, s);
  F.urp.download(rp.data(), n + 1, s);
  F.uci.download(ci.data(), nnz, s);
  F.uv.download(v.data(), nnz, s);
  RCHOL_CUDA(cudaStreamSynchronize(s));
  build_dir_streams(rp, ci, v, n, F.nodes, true, fp32, fmt_mode, kwidth, bwd, s);
}

void build_streams(const rchol_factor_s &F, SolvePlan &P, cudaStream_t s) {
  build_streams_width(F, 1, P.sfwd, P.sbwd, s);
}

// The multi-right-hand-side streams, built on first use.
void build_streams_k(const rchol_factor_s &F, SolvePlan &P, cudaStream_t s) {
  if (P.kbuilt) return;
  build_streams_width(F, KW, P.kfwd, P.kbwd, s);
  if (F.precision == RCHOL_PREC_FP32) P.acck32.alloc((size_t)F.n * KW);
  else P.acck64.alloc((size_t)F.n * KW);
  P.kbuilt = true;
}

// ---- launch ------------------------------------------------------------------------------

constexpr int kMaxDevices = 128;

// A kernel's dynamic shared-memory limit above 48 KiB is an attribute of the
// current device: `set` runs once per device ordinal (per flag array, i.e.
// per kernel family), and concurrent first calls from several host threads
// wait for the one that sets it.  A `set` that throws leaves the flag unset.
template <typename Fn>
static void once_per_device(std::once_flag (&flags)[kMaxDevices], Fn &&set) {
  int dev = 0;
  RCHOL_CUDA(cudaGetDevice(&dev));
  RCHOL_CHECK_ARG(dev >= 0 && dev < kMaxDevices, "device ordinal out of range");
  std::call_once(flags[dev], std::forward<Fn>(set));
}

// External sums of one stage: acc_i = in_i - sum of row i's entries outside
// its piece, for the stage's rows (1, 4, 8 or 32 lanes per row).
template <typename VT, typename InT, typename OutT>
static void launch_ext(const StreamDir &D, size_t st, const VT *ext_v, const InT *in, const OutT *out, VT *acc,
                       cudaStream_t s) {
  const int64_t r0 = D.stage_row_ptr[st], r1 = D.stage_row_ptr[st + 1], nr = r1 - r0;
  const int lanes = D.stage_ext_lanes[st];
  const unsigned eg = (unsigned)((nr * lanes + 255) / 256);
  switch (lanes) {
    case 1:
      ext_kernel<VT, InT, OutT><<<eg, 256, 0, s>>>(D.srows.p + r0, nr, D.ext_rp.p, D.ext_ci.p, ext_v, in, out, acc);
      break;
    case 4:
      ext_lanes_kernel<VT, InT, OutT, 4><<<eg, 256, 0, s>>>(D.srows.p + r0, nr, D.ext_rp.p, D.ext_ci.p, ext_v, in, out, acc);
      break;
    case 8:
      ext_lanes_kernel<VT, InT, OutT, 8><<<eg, 256, 0, s>>>(D.srows.p + r0, nr, D.ext_rp.p, D.ext_ci.p, ext_v, in, out, acc);
      break;
    default:
      ext_lanes_kernel<VT, InT, OutT, 32><<<eg, 256, 0, s>>>(D.srows.p + r0, nr, D.ext_rp.p, D.ext_ci.p, ext_v, in, out, acc);
      break;
  }
  note_launch();
}

// Records prefetched into L2 ahead of use (0: none); RCHOL_TRSV_PREFETCH
// overrides the plan's choice (experiments only).
static int prefetch_distance(int planned) {
  static const int v = [] {
    const char *e = getenv("RCHOL_TRSV_PREFETCH");
    return e ? std::max(0, std::min(28, atoi(e))) : -1;
  }();
  return std::max(0, std::min(28, v < 0 ? planned : v));
}

template <typename VT, typename InT, typename OutT>
static void launch_streams(const SolvePlan &P, bool upper, const InT *in, OutT *out, VT *acc, cudaStream_t s) {
  const StreamDir &D = upper ? P.sbwd : P.sfwd;
  constexpr bool f64 = sizeof(VT) == 8;
  const VT *ext_v = reinterpret_cast<const VT *>(f64 ? (const void *)D.ext_v64.p : (const void *)D.ext_v32.p);
  static std::once_flag attr_once[kMaxDevices];
  once_per_device(attr_once, [&] {
    RCHOL_CUDA(cudaFuncSetAttribute(w2_kernel<VT, InT, OutT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmemCap));
    RCHOL_CUDA(cudaFuncSetAttribute(w2_kernel<VT, InT, OutT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmemCap));
    RCHOL_CUDA(cudaFuncSetAttribute(pipe_kernel<VT, InT, OutT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmemCap));
    RCHOL_CUDA(cudaFuncSetAttribute(pipe_kernel<VT, InT, OutT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmemCap));
  });
  const int sms = sm_count();
  for (size_t st = 0; st + 1 < D.stage_ptr.size(); ++st) {
    const int pieces = D.stage_ptr[st + 1] - D.stage_ptr[st];
    if (!pieces) continue;
    // stages without external entries read the right-hand side directly
    const VT *src_acc = nullptr;
    if (D.stage_ext[st]) {
      launch_ext<VT, InT, OutT>(D, st, ext_v, in, out, acc, s);
      src_acc = acc;
    }
    const size_t bufbytes = al16((size_t)D.stage_maxrec[st]);
    if (D.stage_fmt[st] == FMT_WARP) {
      W2Args<VT> a;
      a.nodes = D.nodes.p;
      a.node0 = D.stage_ptr[st];
      a.node1 = D.stage_ptr[st + 1];
      a.blocks = D.blocks.p;
      a.blk_off = D.blk_off.p;
      a.acc = src_acc;
      a.nbuf = kW2Ring;
      a.bufbytes = (int)bufbytes;
      a.wmask = (uint32_t)D.stage_window[st] - 1u;
      a.per_warp = (int)w2_warp_bytes<VT>(kW2Ring, bufbytes, (size_t)D.stage_window[st]);
      a.pf = prefetch_distance(P.knobs.w2_pf);
      if (a.pf) a.pf = std::max(a.pf, kW2Ring);  // the offset cache holds records k+NB .. k+NB+63
      if ((size_t)a.per_warp > kSmemCap) throw Error(RCHOL_ERR_INTERNAL, "triangular-solve piece exceeds shared memory");
      int wpb = std::max(1, std::min(std::max(1, std::min(8, P.knobs.w2_wpb)), (int)(kSmemCap / (size_t)a.per_warp)));
      // spread small stages over the SMs rather than packing few blocks
      while (wpb > 1 && (pieces + wpb - 1) / wpb < sms) wpb >>= 1;
      a.wpb = wpb;
      const unsigned grid = (unsigned)((pieces + wpb - 1) / wpb);
      const size_t bytes = (size_t)a.per_warp * wpb;
      if (upper) w2_kernel<VT, InT, OutT, true><<<grid, 32 * wpb, bytes, s>>>(a, in, out);
      else w2_kernel<VT, InT, OutT, false><<<grid, 32 * wpb, bytes, s>>>(a, in, out);
    } else {
      PipeArgs<VT> a;
      a.nodes = D.nodes.p;
      a.node0 = D.stage_ptr[st];
      a.blocks = D.blocks.p;
      a.blk_off = D.blk_off.p;
      a.acc = src_acc;
      a.maxchunk = D.stage_chunks[st];
      a.pf = prefetch_distance(pieces <= sms ? P.knobs.pipe_pf : 0);
      const int warps = D.stage_warps[st];
      // every piece takes the deepest ring up to the knob that fits its own
      // rows and records; the launch has the largest of their shared memory
      a.ring = std::max(kPipeRingMin, std::min(kPipeRingMax, P.knobs.pipe_ring));
      const size_t bytes = (size_t)D.stage_smem[st][a.ring];
      a.smem = (int)bytes;
      if (bytes > kSmemCap) throw Error(RCHOL_ERR_INTERNAL, "triangular-solve piece exceeds shared memory");
      const unsigned threads = 32u * (unsigned)warps;
      if (upper) pipe_kernel<VT, InT, OutT, true><<<pieces, threads, bytes, s>>>(a, in, out);
      else pipe_kernel<VT, InT, OutT, false><<<pieces, threads, bytes, s>>>(a, in, out);
    }
    note_launch();
    RCHOL_CUDA(cudaGetLastError());
  }
}

// ---- status of the bounded waits ------------------------------------------------------------

namespace {
// One thread waits on an mbarrier that nothing arrives at, for `polls` polls,
// and records the timeout like the solve kernels do: the path a failed
// record copy takes, exercised without a fault.
__global__ void wait_selftest_kernel(uint32_t polls) {
  __shared__ uint64_t bar;
  if (threadIdx.x != 0) return;
  mbar_init(&bar, 1);
  fence_mbar_init();
  bool done = false;
  for (uint32_t i = 0; i < polls && !done; ++i) done = mbar_test(&bar, 0);
  if (!done) atomicOr(&g_solve_status, 1u);
}
}  // namespace

uint32_t take_solve_status(cudaStream_t s) {
  RCHOL_CUDA(cudaStreamSynchronize(s));
  uint32_t v = 0;
  RCHOL_CUDA(cudaMemcpyFromSymbol(&v, g_solve_status, sizeof(v)));
  if (v) {
    const uint32_t zero = 0;
    RCHOL_CUDA(cudaMemcpyToSymbol(g_solve_status, &zero, sizeof(zero)));
  }
  return v;
}

void check_solve_status(cudaStream_t s) {
  const uint32_t v = take_solve_status(s);
  if (v & 1u) throw Error(RCHOL_ERR_TIMEOUT, "a triangular-solve kernel gave up waiting for a record copy");
  if (v) throw Error(RCHOL_ERR_INTERNAL, "a triangular-solve piece did not fit its launch's shared memory");
}

void wait_selftest(uint32_t polls, cudaStream_t s) {
  wait_selftest_kernel<<<1, 32, 0, s>>>(polls);
  note_launch();
  RCHOL_CUDA(cudaGetLastError());
}

// ---- autotuning of the launch-time choices -----------------------------------------------

std::pair<double, double> tune_solves(const rchol_factor_s &F, SolvePlan &P, cudaStream_t s) {
  const int64_t n = F.n;
  const bool fp32 = F.precision == RCHOL_PREC_FP32;
  DevBuf<double> r(n), z(n), y64(fp32 ? 0 : n);
  DevBuf<float> y32(fp32 ? n : 0);
  if (fp32) {
    if (P.acc32.n < (size_t)n) P.acc32.alloc(n);
  } else if (P.acc64.n < (size_t)n) {
    P.acc64.alloc(n);
  }
  RCHOL_CUDA(cudaMemsetAsync(r.p, 0, r.bytes(), s));
  cudaEvent_t e0, e1;
  RCHOL_CUDA(cudaEventCreate(&e0));
  RCHOL_CUDA(cudaEventCreate(&e1));
  auto apply = [&] {
    if (fp32) {
      launch_streams<float, double, float>(P, false, r.p, y32.p, P.acc32.p, s);
      launch_streams<float, float, double>(P, true, y32.p, z.p, P.acc32.p, s);
    } else {
      launch_streams<double, double, double>(P, false, r.p, y64.p, P.acc64.p, s);
      launch_streams<double, double, double>(P, true, y64.p, z.p, P.acc64.p, s);
    }
  };
  auto time_ms = [&] {
    apply();  // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 3; ++rep) {
      RCHOL_CUDA(cudaEventRecord(e0, s));
      apply();
      RCHOL_CUDA(cudaEventRecord(e1, s));
      RCHOL_CUDA(cudaEventSynchronize(e1));
      float ms = 0.f;
      RCHOL_CUDA(cudaEventElapsedTime(&ms, e0, e1));
      best = std::min(best, ms);
    }
    return (double)best;
  };
  const double before = time_ms();
  double best = before;
  // coordinate descent over the knobs, each from the current best
  auto try_knob = [&](int SolveKnobs::*field, std::initializer_list<int> values) {
    const int keep = P.knobs.*field;
    int pick = keep;
    for (int v : values) {
      if (v == keep) continue;
      P.knobs.*field = v;
      const double ms = time_ms();
      if (ms < best * 0.995) {
        best = ms;
        pick = v;
      }
    }
    P.knobs.*field = pick;
  };
  try_knob(&SolveKnobs::pipe_pf, {0, 8, 16, 24});
  try_knob(&SolveKnobs::pipe_ring, {5, 6, 8});
  try_knob(&SolveKnobs::w2_wpb, {1, 2, 4, 8});
  try_knob(&SolveKnobs::w2_pf, {0, 8, 16});
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // captured PCG iterations launched with the old choices
  P.pcg.clear();
  P.seg.clear();
  P.tuned_ms = best;
  return {before, best};
}

void stream_trsv(const rchol_factor_s &F, const SolvePlan &P, bool upper, const double *in64,
                 const float *in32, double *out64, float *out32, cudaStream_t s) {
  SolvePlan &Pm = const_cast<SolvePlan &>(P);
  const int64_t n = F.n;
  if (F.precision == RCHOL_PREC_FP32) {
    if (Pm.acc32.n < (size_t)n) Pm.acc32.alloc(n);
    if (in64 && out32) launch_streams<float, double, float>(P, upper, in64, out32, Pm.acc32.p, s);
    else if (in32 && out64) launch_streams<float, float, double>(P, upper, in32, out64, Pm.acc32.p, s);
    else if (in64 && out64) launch_streams<float, double, double>(P, upper, in64, out64, Pm.acc32.p, s);
    else throw Error(RCHOL_ERR_INTERNAL, "unsupported triangular-solve operand types");
  } else {
    if (Pm.acc64.n < (size_t)n) Pm.acc64.alloc(n);
    if (in64 && out64) launch_streams<double, double, double>(P, upper, in64, out64, Pm.acc64.p, s);
    else throw Error(RCHOL_ERR_INTERNAL, "unsupported triangular-solve operand types");
  }
}

template <typename VT, typename InT, typename OutT>
static void launch_streams_k(const SolvePlan &P, bool upper, const InT *in, OutT *out, VT *acc, int k,
                             int64_t ld, cudaStream_t s) {
  const StreamDir &D = upper ? P.kbwd : P.kfwd;
  constexpr bool f64 = sizeof(VT) == 8;
  const VT *ext_v = reinterpret_cast<const VT *>(f64 ? (const void *)D.ext_v64.p : (const void *)D.ext_v32.p);
  const int smem_cap = 220 * 1024;
  static std::once_flag attr_once[kMaxDevices];
  once_per_device(attr_once, [&] {
    RCHOL_CUDA(cudaFuncSetAttribute(team_k_kernel<VT, OutT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    smem_cap));
    RCHOL_CUDA(cudaFuncSetAttribute(team_k_kernel<VT, OutT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    smem_cap));
  });
  TeamArgs<VT> ta;
  ta.nodes = D.nodes.p;
  ta.blocks = D.blocks.p;
  ta.blk_off = D.blk_off.p;
  ta.acc = acc;
  ta.maxchunk = 0;
  for (size_t st = 0; st + 1 < D.stage_ptr.size(); ++st) {
    const int pieces = D.stage_ptr[st + 1] - D.stage_ptr[st];
    if (!pieces) continue;
    const int64_t r0 = D.stage_row_ptr[st], r1 = D.stage_row_ptr[st + 1], nr = r1 - r0;
    ext_k_kernel<VT, InT, OutT><<<(unsigned)((nr * 32 + 255) / 256), 256, 0, s>>>(
        D.srows.p + r0, nr, D.ext_rp.p, D.ext_ci.p, ext_v, in, out, acc, k, ld);
    note_launch();
    ta.node0 = D.stage_ptr[st];
    // every piece takes the deepest ring up to this one that fits its own
    // rows and records; the launch has the largest of their shared memory
    ta.ring = pieces > 2 * sm_count() ? 5 : TEAM_RING_MAX;
    const size_t bytes = (size_t)D.stage_smem[st][ta.ring];
    ta.smem = (int)bytes;
    if (bytes > (size_t)smem_cap) throw Error(RCHOL_ERR_INTERNAL, "triangular-solve piece exceeds shared memory");
    if (upper) team_k_kernel<VT, OutT, true><<<pieces, 256, bytes, s>>>(ta, out, k, ld);
    else team_k_kernel<VT, OutT, false><<<pieces, 256, bytes, s>>>(ta, out, k, ld);
    note_launch();
    RCHOL_CUDA(cudaGetLastError());
  }
}

void stream_trsv_k(const rchol_factor_s &F, const SolvePlan &P, bool upper, const double *in64,
                   const float *in32, double *out64, float *out32, int k, cudaStream_t s) {
  if (!P.kbuilt) throw Error(RCHOL_ERR_INTERNAL, "multi-right-hand-side streams not built");
  for (int j0 = 0; j0 < k; j0 += KW) {  // groups of up to KW columns
    const int kg = std::min(KW, k - j0);
    if (F.precision == RCHOL_PREC_FP32) {
      float *acc = P.acck32.p;
      if (in64 && out32) launch_streams_k<float, double, float>(P, upper, in64 + j0, out32 + j0, acc, kg, k, s);
      else if (in32 && out64) launch_streams_k<float, float, double>(P, upper, in32 + j0, out64 + j0, acc, kg, k, s);
      else if (in64 && out64) launch_streams_k<float, double, double>(P, upper, in64 + j0, out64 + j0, acc, kg, k, s);
      else throw Error(RCHOL_ERR_INTERNAL, "unsupported triangular-solve operand types");
    } else {
      if (in64 && out64)
        launch_streams_k<double, double, double>(P, upper, in64 + j0, out64 + j0, P.acck64.p, kg, k, s);
      else throw Error(RCHOL_ERR_INTERNAL, "unsupported triangular-solve operand types");
    }
  }
}

// ---- preconditioner apply without allocation --------------------------------------------
//
// Some callers cannot allocate device memory at solve time: code that runs
// under a fixed memory budget decided at start-up, allocator-free real-time
// loops, or hosts that own all device memory themselves.  For them the
// preconditioner z = (G G^T)^-1 r can run with its two scratch vectors (the
// partial sums and the intermediate y = G^-1 r) in this fixed, file-scope
// device array instead of buffers allocated with the factor's plan.  Every
// GPU that loads the library holds the array until the process exits.
// The array is shared by all calls and keeps the last call's contents; nothing
// in it has to start at zero (both vectors are fully written before they are
// read), and calls that overlap on the GPU race on it.
constexpr size_t kNoAllocScratchBytes = size_t(16) << 20;  // 16 MiB
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

namespace {
std::mutex g_noalloc_mutex;
void *g_noalloc_ptr[kMaxDevices] = {};  // device address of the array, per device ordinal
}  // namespace

size_t noalloc_scratch_bytes() { return kNoAllocScratchBytes; }

// Set-up on the current device: the array's host-side name is only a
// stand-in, so its device address is looked up with the device current.  The
// first call on a device does this (it should come before any stream
// capture); later calls whose stream is not capturing look it up again, so a
// device reset (which gives the array a new address) leaves no stale pointer.
static void *noalloc_scratch_address(cudaStream_t s) {
  int dev = 0;
  RCHOL_CUDA(cudaGetDevice(&dev));
  RCHOL_CHECK_ARG(dev >= 0 && dev < kMaxDevices, "device ordinal out of range");
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
    (void)cudaGetLastError();  // e.g. the legacy stream while another stream captures
    cs = cudaStreamCaptureStatusActive;
  }
  std::lock_guard<std::mutex> guard(g_noalloc_mutex);
  if (!g_noalloc_ptr[dev] || cs == cudaStreamCaptureStatusNone) {
    void *p = nullptr;
    RCHOL_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    g_noalloc_ptr[dev] = p;
  }
  return g_noalloc_ptr[dev];
}

void precond_noalloc(const rchol_factor_s &F, const double *r, double *z, cudaStream_t s) {
  const int64_t n = F.n;
  const bool fp32 = F.precision == RCHOL_PREC_FP32;
  const size_t vsz = fp32 ? 4 : 8;
  const size_t acc_bytes = al16((size_t)n * vsz);
  if (2 * acc_bytes > kNoAllocScratchBytes)
    throw Error(RCHOL_ERR_INVALID, "n = " + std::to_string(n) + " needs " + std::to_string(2 * acc_bytes) +
                                       " bytes of scratch; the allocation-free entry point has " +
                                       std::to_string(kNoAllocScratchBytes) + " (n <= " +
                                       std::to_string(kNoAllocScratchBytes / (2 * vsz)) + " for this precision)");
  unsigned char *base = static_cast<unsigned char *>(noalloc_scratch_address(s));
  const SolvePlan &P = *F.plan;
  if (fp32) {
    float *acc = reinterpret_cast<float *>(base);
    float *y = reinterpret_cast<float *>(base + acc_bytes);
    launch_streams<float, double, float>(P, false, r, y, acc, s);
    launch_streams<float, float, double>(P, true, y, z, acc, s);
  } else {
    double *acc = reinterpret_cast<double *>(base);
    double *y = reinterpret_cast<double *>(base + acc_bytes);
    launch_streams<double, double, double>(P, false, r, y, acc, s);
    launch_streams<double, double, double>(P, true, y, z, acc, s);
  }
}

}  // namespace rchol
