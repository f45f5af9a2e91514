// Dense-block triangular solves with G (forward) and G^T (backward).
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
// forward solve, root first for the backward one).  A node larger than shared
// memory is cut into pieces solved one after another.  Per stage:
//   ext_kernel    acc_i = rhs_i - sum of row i's entries outside its piece
//                 (columns already solved), all SMs; 1, 4, 8 or 32 lanes per
//                 row (ext_lanes_kernel) by the stage's mean row length.
//   team_kernel   one thread block per piece (default): the piece's unknowns
//                 live in shared memory, block records stream in through a
//                 cp.async ring; warp 0 solves block k (near entries from the
//                 previous block by shuffles, then the dense inverse) while
//                 the helper warps sum the far entries of block k + 1:
//                   t_r = acc_r - sum_{earlier blocks} G_rj x_j   (sparse)
//                   x_r = sum_c (T^-1)_{rc} t_c                   (dense, 32 shuffles)
//   block_kernel  one warp per piece, the same arithmetic without helpers
//                 (depths whose blocks are too dense for the team ring).
// Values are FP32 or FP64 as the factor is stored; the block inverses are
// computed in FP64 on the host and rounded to the stored precision.

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

void build_piece(const std::vector<int64_t> &rp, const std::vector<int32_t> &ci, const std::vector<double> &v,
                 int64_t b, int64_t e, bool upper, size_t vsz, PieceBuild &P) {
  const int64_t R = e - b, nb = (R + BS - 1) / BS;
  const size_t csz = R > 65535 ? 4 : 2;
  P.offs.assign(1, 0);
  P.bytes.clear();
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
        if (lc >= row0 && lc < row0 + nr) {
          T[r][lc - row0] = v[q];  // inside the block (diagonal included)
        } else {
          cols[r].push_back((uint32_t)lc);
          vals[r].push_back(v[q]);
          ++nent;
        }
      }
    }
    invert_block(T, upper, X);
    // record layout
    const size_t o_off = 16, o_col = o_off + al16(4 * (BS + 1)), o_val = o_col + al16(csz * nent),
                 o_min = o_val + al16(vsz * nent), len = o_min + al16(vsz * TRI);
    const size_t base = P.bytes.size();
    P.bytes.resize(base + len, 0);
    unsigned char *p = P.bytes.data() + base;
    uint32_t hdr[4] = {(uint32_t)nr, nent, (uint32_t)row0, (uint32_t)csz};
    std::memcpy(p, hdr, 16);
    uint32_t off[BS + 1];
    off[0] = 0;
    for (int r = 0; r < BS; ++r) off[r + 1] = off[r] + (uint32_t)cols[r].size();
    std::memcpy(p + o_off, off, 4 * (BS + 1));
    size_t w = 0;
    for (int r = 0; r < BS; ++r)
      for (size_t t = 0; t < cols[r].size(); ++t, ++w) {
        if (csz == 2) {
          uint16_t c16 = (uint16_t)cols[r][t];
          std::memcpy(p + o_col + 2 * w, &c16, 2);
        } else {
          std::memcpy(p + o_col + 4 * w, &cols[r][t], 4);
        }
        if (vsz == 8) std::memcpy(p + o_val + 8 * w, &vals[r][t], 8);
        else {
          float f = (float)vals[r][t];
          std::memcpy(p + o_val + 4 * w, &f, 4);
        }
      }
    for (int c = 0; c < BS; ++c) {
      const int r_lo = upper ? 0 : c, r_hi = upper ? c : BS - 1;
      for (int r = r_lo; r <= r_hi; ++r) {
        const double m = (r < nr && c < nr) ? X[r][c] : 0.0;
        const size_t at = (size_t)tri_col_off(c, upper) + (size_t)(r - r_lo);
        if (vsz == 8) std::memcpy(p + o_min + 8 * at, &m, 8);
        else {
          float f = (float)m;
          std::memcpy(p + o_min + 4 * at, &f, 4);
        }
      }
    }
    P.offs.push_back((int64_t)P.bytes.size());
    P.maxrec = std::max<int32_t>(P.maxrec, (int32_t)len);
    P.sparse += nent;
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

template <typename VT>
struct BlockArgs {
  const NodeDesc *nodes;
  int node0, node1;     // pieces of this stage
  int wpb;              // warps (pieces) per thread block
  int bufbytes;         // per-buffer bytes (16-aligned)
  int nbuf;             // block records in flight per warp (ring of buffers), 2..6
  int per_warp;         // shared-memory bytes per warp
  bool upper;           // backward solve: upper-triangular block inverses
  const unsigned char *blocks;
  const int64_t *blk_off;
  const VT *acc;
};

template <typename VT, typename OutT, bool UPPER>
__global__ void __launch_bounds__(128) block_kernel(BlockArgs<VT> a, OutT *out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int piece = a.node0 + blockIdx.x * a.wpb + w;
  if (piece >= a.node1) return;  // the whole warp leaves
  const NodeDesc nd = a.nodes[piece];
  unsigned char *base = smem + (size_t)w * a.per_warp;
  const int nbuf = a.nbuf;
  VT *xs = reinterpret_cast<VT *>(base + (size_t)nbuf * a.bufbytes);
  const unsigned char *src = a.blocks;
  const int64_t *boff = a.blk_off + nd.blk0;

  // ring of nbuf block buffers; block k lives in slot k % nbuf
  auto load = [&](int k) {
    unsigned char *dst = base + (size_t)(k % nbuf) * a.bufbytes;
    const int64_t o0 = boff[k];
    int64_t len = boff[k + 1] - o0;
#ifdef RCHOL_DEVICE_CHECKS
    if (len < 0 || len > a.bufbytes || (o0 & 15)) {
      if (lane == 0) dbg_report("block record length", len, a.bufbytes);
      len = 0;
    }
#endif
    for (int64_t o = lane * 16; o < len; o += 32 * 16) cp_async16(dst + o, src + o0 + o);
    cp_async_commit();
  };
#ifdef RCHOL_DEVICE_CHECKS
  if ((int64_t)nbuf * a.bufbytes + (int64_t)nd.rows * (int64_t)sizeof(VT) > a.per_warp ||
      nd.begin < 0 || nd.begin + nd.rows > dbg_n) {
    if (lane == 0) dbg_report("piece layout (rows)", nd.rows, a.per_warp);
    return;
  }
#endif
  for (int k = 0; k < nbuf - 1 && k < nd.nblocks; ++k) load(k);
  for (int r = lane; r < nd.rows; r += 32) xs[r] = a.acc[nd.begin + r];
  __syncwarp();

  for (int k = 0; k < nd.nblocks; ++k) {
    // refill the slot block k-1 used (finished last step), then wait for block
    // k; the groups committed after block k's may stay in flight
    if (k + nbuf - 1 < nd.nblocks) load(k + nbuf - 1);
    const int after = min(nbuf - 1, nd.nblocks - 1 - k);
    switch (after) {
      case 0: cp_async_wait<0>(); break;
      case 1: cp_async_wait<1>(); break;
      case 2: cp_async_wait<2>(); break;
      case 3: cp_async_wait<3>(); break;
      case 4: cp_async_wait<4>(); break;
      default: cp_async_wait<5>(); break;
    }
    __syncwarp();
    const unsigned char *p = base + (size_t)(k % nbuf) * a.bufbytes;
    const uint32_t *hdr = reinterpret_cast<const uint32_t *>(p);
    const uint32_t nr = hdr[0], nent = hdr[1], row0 = hdr[2], csz = hdr[3];
    const uint32_t *eoff = reinterpret_cast<const uint32_t *>(p + 16);
    const size_t o_col = 16 + al16(4 * (BS + 1));
    const size_t o_val = o_col + al16((size_t)csz * nent);
    const size_t o_min = o_val + al16(sizeof(VT) * nent);
    const VT *val = reinterpret_cast<const VT *>(p + o_val);
    const VT *minv = reinterpret_cast<const VT *>(p + o_min);
#ifdef RCHOL_DEVICE_CHECKS
    if (nr > (uint32_t)BS || (int64_t)row0 + nr > nd.rows || (csz != 2 && csz != 4) || eoff[BS] != nent ||
        (int64_t)(o_min + sizeof(VT) * TRI) > a.bufbytes) {
      if (lane == 0) dbg_report("block header (row0)", row0, nd.rows);
      return;
    }
    bool badc = false;
    for (uint32_t e = eoff[lane]; e < eoff[lane + 1]; ++e) {
      const uint32_t cc = csz == 2 ? reinterpret_cast<const uint16_t *>(p + o_col)[e]
                                   : reinterpret_cast<const uint32_t *>(p + o_col)[e];
      if (cc >= (uint32_t)nd.rows) {
        dbg_report("block column", cc, nd.rows);
        badc = true;
      }
    }
    if (__any_sync(0xffffffffu, badc)) return;
#endif
    VT t = 0;
    if (lane < (int)nr) {
      VT s0 = 0, s1 = 0;
      uint32_t e = eoff[lane];
      const uint32_t e1 = eoff[lane + 1];
      if (csz == 2) {
        const uint16_t *col = reinterpret_cast<const uint16_t *>(p + o_col);
        for (; e + 1 < e1; e += 2) {
          s0 += val[e] * xs[col[e]];
          s1 += val[e + 1] * xs[col[e + 1]];
        }
        if (e < e1) s0 += val[e] * xs[col[e]];
      } else {
        const uint32_t *col = reinterpret_cast<const uint32_t *>(p + o_col);
        for (; e + 1 < e1; e += 2) {
          s0 += val[e] * xs[col[e]];
          s1 += val[e + 1] * xs[col[e + 1]];
        }
        if (e < e1) s0 += val[e] * xs[col[e]];
      }
      t = xs[row0 + lane] - (s0 + s1);
    }
    // x_lane = sum_c Minv[lane][c] t_c over the stored triangle
    VT c0 = 0, c1 = 0, c2 = 0, c3 = 0;
    auto term = [&](int c) -> VT {
      const VT tc = __shfl_sync(0xffffffffu, t, c);
      const bool in = UPPER ? (lane <= c) : (lane >= c);
      const int at = tri_col_off(c, UPPER) + (UPPER ? lane : lane - c);
      return in ? minv[at] * tc : VT(0);
    };
#pragma unroll
    for (int c = 0; c < BS; c += 4) {
      c0 += term(c + 0);
      c1 += term(c + 1);
      c2 += term(c + 2);
      c3 += term(c + 3);
    }
    if (lane < (int)nr) xs[row0 + lane] = (c0 + c1) + (c2 + c3);
    __syncwarp();
  }
  __syncwarp();
  for (int r = lane; r < nd.rows; r += 32) out[nd.begin + r] = (OutT)xs[r];
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

template <typename VT>
struct TeamArgs {
  const NodeDesc *nodes;
  int node0;            // first piece of the stage; piece = node0 + blockIdx.x
  int bufbytes;         // per-record buffer (16-aligned)
  int ring;             // records in the ring (4..8): the solved block's, the next one's, ring-2 in flight
  int maxchunk;         // most chunks of one block (chunk-sum buffer)
  const unsigned char *blocks;
  const int64_t *blk_off;
  const VT *acc;
};

constexpr int TEAM_RING = 4;  // ring used to cut pieces; launches deepen it where room is left (3 at least)
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

// Sum of chunk c: clen entries interleaved with stride nchunk.
template <typename VT, typename CT>
__device__ __forceinline__ VT chunk_sum(const CT *col, const VT *val, const VT *x, uint32_t c, uint32_t nchunk,
                                        uint32_t clen) {
  VT s0 = 0, s1 = 0;
  uint32_t j = 0, at = c;
  for (; j + 1 < clen; j += 2, at += 2 * nchunk) {
    s0 += val[at] * x[col[at]];
    s1 += val[at + nchunk] * x[col[at + nchunk]];
  }
  if (j < clen) s0 += val[at] * x[col[at]];
  return s0 + s1;
}

// Named barrier of the helper warps only (the solver does not take part).
__device__ __forceinline__ void helpers_sync(int nthreads) {
  asm volatile("bar.sync 1, %0;\n" ::"r"(nthreads) : "memory");
}

// One thread block per piece.  Per step k (one __syncthreads):
//   warp 0   t = u_k - near_k . x_{k-1} (shuffles of the previous block's
//            solution, kept in registers), x_k = T_k^-1 t (shuffles);
//   helpers  chunk sums of block k+1 (columns solved before block k), then
//            warp 1 folds them per row into u_{k+1} = acc - far; all helper
//            threads stream record k+RING-1 into the ring.
// The solver's chain per step is therefore only shuffles and FMAs; every
// load it issues is independent of the previous block.
template <typename VT, typename OutT, bool UPPER>
__global__ void __launch_bounds__(256, 2) team_kernel(TeamArgs<VT> a, OutT *out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const NodeDesc nd = a.nodes[a.node0 + blockIdx.x];
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int ht = tid - 32, TH = (int)blockDim.x - 32;  // helper thread index / count
  unsigned char *ring = smem;
  const int RING = a.ring;
  VT *part = reinterpret_cast<VT *>(smem + (size_t)RING * a.bufbytes);  // chunk sums of the next block
  VT *ubuf = reinterpret_cast<VT *>(reinterpret_cast<unsigned char *>(part) + al16((size_t)a.maxchunk * sizeof(VT)));
  VT *xs = ubuf + 2 * BS;  // u of blocks k and k+1 (parity), then the piece's unknowns
  const unsigned char *src = a.blocks;
  const int64_t *boff = a.blk_off + nd.blk0;
  const int nb = nd.nblocks;

  auto load = [&](int k, int slot) {  // helpers only; one commit group per record (empty past the end)
    if (k < nb) {
      unsigned char *dst = ring + (size_t)slot * a.bufbytes;
      const int64_t o0 = boff[k], len = boff[k + 1] - o0;
      for (int64_t o = (int64_t)ht * 16; o < len; o += (int64_t)TH * 16) cp_async16(dst + o, src + o0 + o);
    }
    cp_async_commit();
  };
  for (int r = tid; r < nd.rows; r += blockDim.x) xs[r] = a.acc[nd.begin + r];
  if (warp > 0) {
    for (int k = 0; k < RING - 1; ++k) load(k, k);
    cp_async_wait_upto(RING - 3);  // records 0 and 1 are in
  }
  __syncthreads();

  VT xprev = 0;  // solver: x of the previous block, lane c = its row c
  int slot = 0;  // ring slot of record k
  for (int k = 0; k < nb; ++k) {
    const int next = slot + 1 == RING ? 0 : slot + 1;
    if (warp == 0) {
      const unsigned char *p = ring + (size_t)slot * a.bufbytes;
      const TeamHdr h = read_hdr(p);
      const VT *minv = reinterpret_cast<const VT *>(p + h.o_min);
      // the lane's row of the inverse (zero outside the triangle)
      VT m[BS];
#pragma unroll
      for (int c = 0; c < BS; ++c) {
        const bool in = UPPER ? (lane <= c) : (lane >= c);
        m[c] = minv[in ? tri_col_off(c, UPPER) + (UPPER ? lane : lane - c) : 0];
        m[c] = in ? m[c] : VT(0);
      }
      const bool row = lane < (int)h.nr;
      // u = acc - far (block 0 has no far entries)
      const VT u = !row ? VT(0) : k == 0 ? xs[h.row0 + lane] : ubuf[(k & 1) * BS + lane];
      const uint16_t *noff = reinterpret_cast<const uint16_t *>(p + h.o_noff);
      const unsigned char *ncol = p + h.o_ncol;
      const VT *nval = reinterpret_cast<const VT *>(p + h.o_nval);
      const uint32_t e0 = noff[lane], cnt = row ? noff[lane + 1] - e0 : 0;
      VT s0 = 0, s1 = 0;
      uint32_t j = 0;
      for (; j + 1 < h.nmax; j += 2) {  // uniform trip count: every lane takes part in the shuffles
        const bool ok0 = j < cnt, ok1 = j + 1 < cnt;
        const int c0 = ok0 ? ncol[e0 + j] : 0, c1 = ok1 ? ncol[e0 + j + 1] : 0;
        const VT v0 = ok0 ? nval[e0 + j] : VT(0), v1 = ok1 ? nval[e0 + j + 1] : VT(0);
        s0 += v0 * __shfl_sync(0xffffffffu, xprev, c0);
        s1 += v1 * __shfl_sync(0xffffffffu, xprev, c1);
      }
      if (j < h.nmax) {
        const bool ok0 = j < cnt;
        const int c0 = ok0 ? ncol[e0 + j] : 0;
        const VT v0 = ok0 ? nval[e0 + j] : VT(0);
        s0 += v0 * __shfl_sync(0xffffffffu, xprev, c0);
      }
      const VT t = u - (s0 + s1);
      VT d0 = 0, d1 = 0, d2 = 0, d3 = 0;
#pragma unroll
      for (int c = 0; c < BS; c += 4) {
        d0 += m[c + 0] * __shfl_sync(0xffffffffu, t, c + 0);
        d1 += m[c + 1] * __shfl_sync(0xffffffffu, t, c + 1);
        d2 += m[c + 2] * __shfl_sync(0xffffffffu, t, c + 2);
        d3 += m[c + 3] * __shfl_sync(0xffffffffu, t, c + 3);
      }
      const VT x = (d0 + d1) + (d2 + d3);
      if (row) xs[h.row0 + lane] = x;
      xprev = x;
    } else {
      if (k + 1 < nb) {  // block k+1: far sums (columns solved before block k), then u per row
        const unsigned char *p = ring + (size_t)next * a.bufbytes;
        const TeamHdr h = read_hdr(p);
        const VT *fval = reinterpret_cast<const VT *>(p + h.o_fval);
        for (int c = ht; c < (int)h.nchunk; c += TH)
          part[c] = h.csz == 2 ? chunk_sum(reinterpret_cast<const uint16_t *>(p + h.o_fcol), fval, xs, c, h.nchunk, h.clen)
                               : chunk_sum(reinterpret_cast<const uint32_t *>(p + h.o_fcol), fval, xs, c, h.nchunk, h.clen);
        helpers_sync(TH);
        if (ht < BS) {
          const uint16_t *crow = reinterpret_cast<const uint16_t *>(p + h.o_crow);
          VT f0 = 0, f1 = 0;
          uint32_t c = crow[ht];
          const uint32_t c1 = crow[ht + 1];
          for (; c + 1 < c1; c += 2) {
            f0 += part[c];
            f1 += part[c + 1];
          }
          if (c < c1) f0 += part[c];
          ubuf[((k + 1) & 1) * BS + ht] = ht < (int)h.nr ? xs[h.row0 + ht] - (f0 + f1) : VT(0);
        }
      }
      // record k+RING-1 goes into the slot of record k-1, retired last step
      load(k + RING - 1, slot == 0 ? RING - 1 : slot - 1);
      cp_async_wait_upto(RING - 3);  // records up to k+2 are in
    }
    slot = next;
    __syncthreads();
  }
  for (int r = tid; r < nd.rows; r += blockDim.x) out[nd.begin + r] = (OutT)xs[r];
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
  const int RING = a.ring;
  unsigned char *ring = smem;
  VT *part = reinterpret_cast<VT *>(smem + (size_t)RING * a.bufbytes);  // [2][BS][KW]
  VT *xs = part + 2 * BS * KW;                                           // [rows][KW]
  const unsigned char *src = a.blocks;
  const int64_t *boff = a.blk_off + nd.blk0;
  const int nb = nd.nblocks;

  auto load = [&](int b) {
    if (b < nb) {
      unsigned char *dst = ring + (size_t)(b % RING) * a.bufbytes;
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
      const unsigned char *p = ring + (size_t)(b % RING) * a.bufbytes;
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
        const unsigned char *p = ring + (size_t)((b + 1) % RING) * a.bufbytes;
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

}  // namespace

// ---- plan construction ---------------------------------------------------------------

// SM count of the current device (a scheduling heuristic only: without a
// device, as in host-side plan checks, the GB300's 152 is assumed).
static int sm_count() {
  static int count = 0;
  if (!count) {
    int dev = 0, c = 0;
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&c, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && c > 0)
      count = c;
    else
      count = 152;
  }
  return count;
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
  std::vector<int> stage_team;
};

static void build_dir_streams(const std::vector<int64_t> &rp, const std::vector<int32_t> &ci,
                              const std::vector<double> &v, int64_t n, const std::vector<TreeNode> &tnodes,
                              bool upper, bool fp32, int team_mode, int kwidth, StreamDir &D, cudaStream_t s,
                              HostStreamCopy *host_copy = nullptr) {
  const size_t vsz = fp32 ? 4 : 8;
  const size_t row_bytes = vsz * (size_t)kwidth;  // a piece's unknowns per row in shared memory
  if (kwidth > 1) team_mode = 2;                  // several right-hand sides: team format only
  // Pieces: a node is cut into consecutive pieces (whole blocks) so that the
  // shared memory of its solver holds the piece's unknowns plus its record
  // buffers: two for the warp format (more at launch where room is left),
  // the ring and the chunk sums for the team format.  The bound of a block
  // record counts every entry of its rows that lies in the node but outside
  // the block (an upper bound of its sparse part).
  const size_t budget = 200 * 1024;
  int maxdepth = 1;
  for (auto &nd : tnodes) maxdepth = std::max(maxdepth, nd.depth);
  // One team size for all depths: doubling the team where few pieces run
  // measured slower (the extra helpers' barrier and shared-memory traffic
  // cost more than their shorter chunks save).
  auto team_warps_of = [&](int) { return D.team_warps; };
  // team format for separators (few, long chains), warp format for leaves
  auto team_depth = [&](int depth) {
    if (team_mode == 0) return false;
    return team_mode == 2 || depth < maxdepth;
  };
  struct Piece {
    int64_t b, e;
    bool team;
    int warps;
  };
  auto cut_node = [&](int64_t b, int64_t e, bool team, int warps) {
    const int helper_threads = 32 * (warps - 1);
    std::vector<Piece> out;
    const int64_t nb = (e - b + BS - 1) / BS;
    std::vector<size_t> recb(nb);
    parallel_for(nb, [&](int64_t k0, int64_t k1) {
      for (int64_t k = k0; k < k1; ++k) {
        const int64_t r0 = b + k * BS, r1 = std::min(e, r0 + BS);
        size_t cnt = 0;
        for (int64_t i = r0; i < r1; ++i)
          for (int64_t q = rp[i]; q < rp[i + 1]; ++q) cnt += (ci[q] >= b && ci[q] < e && (ci[q] < r0 || ci[q] >= r1));
        recb[k] = team ? team_record_bound(cnt, helper_threads, vsz, e - b > 65535 ? 4 : 2)
                       : 16 + al16(4 * (BS + 1)) + al16(4 * cnt) + al16(vsz * cnt) + al16(vsz * TRI);
      }
    }, 256);
    const size_t fixed = !team ? 0
                         : kwidth > 1 ? 2 * (size_t)BS * KW * vsz
                                      : 2 * al16((size_t)(helper_threads + BS) * vsz);
    const size_t nrec = team ? TEAM_RING : 2;
    int64_t k = 0;
    while (k < nb) {
      int64_t k1 = k;
      size_t mx = 0;
      while (k1 < nb) {
        const size_t m2 = std::max(mx, recb[k1]);
        const int64_t rows = std::min(e, b + (k1 + 1) * BS) - (b + k * BS);
        if (k1 > k && (fixed + nrec * al16(m2) + (size_t)rows * row_bytes > budget || rows > 65535)) break;
        mx = m2;
        ++k1;
      }
      // a single block may run with the smallest ring (3 records: no copy in
      // flight across a step) rather than fall back to the warp format
      const size_t nmin = team ? 3 : 2;
      if (fixed + nmin * al16(mx) + (size_t)(std::min(e, b + k1 * BS) - (b + k * BS)) * row_bytes > budget)
        throw Error(RCHOL_ERR_INTERNAL, "a 32-row block of G is too dense for the shared-memory solve");
      out.push_back(Piece{b + k * BS, std::min(e, b + k1 * BS), team, warps});
      k = k1;
    }
    return out;
  };
  std::vector<Piece> pieces;
  std::vector<char> team_failed(maxdepth + 1, 0);
  D.stage_ptr.assign(1, 0);
  for (int st = 0; st < maxdepth; ++st) {
    const int depth = upper ? st + 1 : maxdepth - st;
    std::vector<std::vector<Piece>> by_index;  // piece j of every node of this depth
    bool retry_depth = false;
    for (auto &nd : tnodes) {
      if (nd.depth != depth) continue;
      const int64_t b = nd.begin, e = std::min(nd.end, n);
      if (e <= b) continue;
      std::vector<Piece> ps;
      bool team = team_depth(depth) && !team_failed[depth];
      try {
        ps = cut_node(b, e, team, team_warps_of(depth));
      } catch (const Error &) {
        if (!team || kwidth > 1) throw;
        // a block too dense for the team ring: this depth uses the warp format
        team_failed[depth] = true;
        retry_depth = true;
        break;
      }
      if (upper) std::reverse(ps.begin(), ps.end());  // backward: last piece first
      if (by_index.size() < ps.size()) by_index.resize(ps.size());
      for (size_t j = 0; j < ps.size(); ++j) by_index[j].push_back(ps[j]);
    }
    if (retry_depth) {
      --st;  // the same depth again, in the warp format
      continue;
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
  // block records
  std::vector<PieceBuild> built(np);
  std::vector<int32_t> chunks(np, 0);
  parallel_for(np, [&](int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; ++k) {
      if (pieces[k].team)
        build_team_piece(rp, ci, v, pieces[k].b, pieces[k].e, upper, vsz, 32 * (pieces[k].warps - 1), kwidth > 1,
                         built[k], chunks[k]);
      else
        build_piece(rp, ci, v, pieces[k].b, pieces[k].e, upper, vsz, built[k]);
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
  std::vector<unsigned char> all(total);
  parallel_for(np, [&](int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; ++k)
      std::memcpy(all.data() + blk_off[desc[k].blk0], built[k].bytes.data(), built[k].bytes.size());
  }, 1);
  built.clear();
  // stages
  D.stage_rows.clear();
  D.stage_maxrec.clear();
  D.stage_team.clear();
  D.stage_warps.clear();
  D.stage_chunks.clear();
  D.stage_ext_lanes.clear();
  D.stage_row_ptr.assign(1, 0);
  D.steps = 0;
  std::vector<int32_t> srows;
  for (size_t st = 0; st + 1 < D.stage_ptr.size(); ++st) {
    int rows = 0, maxrec = 16, steps = 0, maxchunk = 0;
    int64_t ext = 0, nrow = 0;
    for (int k = D.stage_ptr[st]; k < D.stage_ptr[st + 1]; ++k) {
      rows = std::max(rows, desc[k].rows);
      maxrec = std::max(maxrec, desc[k].maxrec);
      steps = std::max(steps, desc[k].nblocks);
      maxchunk = std::max(maxchunk, desc[k].maxchunk);
      for (int64_t i = desc[k].begin; i < desc[k].begin + desc[k].rows; ++i) srows.push_back((int32_t)i);
      ext += ext_rp[desc[k].begin + desc[k].rows] - ext_rp[desc[k].begin];
      nrow += desc[k].rows;
    }
    const bool team = D.stage_ptr[st + 1] > D.stage_ptr[st] && pieces[D.stage_ptr[st]].team;
    const double avg = nrow ? (double)ext / (double)nrow : 0.0;
    D.stage_rows.push_back(rows);
    D.stage_maxrec.push_back(maxrec);
    D.stage_team.push_back(team ? 1 : 0);
    D.stage_warps.push_back(D.stage_ptr[st + 1] > D.stage_ptr[st] ? pieces[D.stage_ptr[st]].warps : D.team_warps);
    D.stage_chunks.push_back(std::max(1, maxchunk));
    D.stage_ext_lanes.push_back(avg < 6 ? 1 : avg < 24 ? 4 : avg < 96 ? 8 : 32);
    D.stage_row_ptr.push_back((int64_t)srows.size());
    D.steps += steps;
  }
  D.nblocks = (int64_t)blk_off.size() - np;
  D.ext_nnz = next;
  if (host_copy) {
    host_copy->blocks.swap(all);
    host_copy->blk_off = blk_off;
    host_copy->desc = desc;
    host_copy->ext_rp = ext_rp;
    host_copy->ext_ci = eci;
    host_copy->ext_v = ev;
    host_copy->stage_ptr = D.stage_ptr;
    host_copy->stage_team = D.stage_team;
    return;
  }
  D.blocks.upload(all.data(), all.size(), s);
  D.blk_off.upload(blk_off.data(), blk_off.size(), s);
  D.nodes.upload(desc.data(), np, s);
  D.ext_rp.upload(ext_rp.data(), n + 1, s);
  D.ext_ci.upload(eci.data(), next, s);
  if (!fp32) D.ext_v64.upload(ev.data(), next, s);
  std::vector<float> ev32;
  if (fp32) {
    ev32.resize(next);
    for (int64_t q = 0; q < next; ++q) ev32[q] = (float)ev[q];
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
  // Schedule knobs (tuning only; every setting solves exactly the same
  // system): RCHOL_TRSV_TEAM = 0 warp format everywhere, 1 team format for
  // separators, 2 team format everywhere (default); RCHOL_TRSV_TEAM_WARPS =
  // warps of a team (2..8, default 8).
  int team_mode = 2, team_warps = 8;
  if (const char *e = getenv("RCHOL_TRSV_TEAM")) team_mode = std::max(0, std::min(2, atoi(e)));
  if (const char *e = getenv("RCHOL_TRSV_TEAM_WARPS")) team_warps = std::max(2, std::min(8, atoi(e)));
  if (kwidth > 1) team_warps = 8;
  fwd.team_warps = bwd.team_warps = team_warps;
  build_dir_streams(rp, ci, v, n, F.nodes, false, fp32, team_mode, kwidth, fwd, s);
  F.urp.download(rp.data(), n + 1, s);
  F.uci.download(ci.data(), nnz, s);
  F.uv.download(v.data(), nnz, s);
  RCHOL_CUDA(cudaStreamSynchronize(s));
  build_dir_streams(rp, ci, v, n, F.nodes, true, fp32, team_mode, kwidth, bwd, s);
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

template <typename VT, typename InT, typename OutT>
static void launch_streams(const SolvePlan &P, bool upper, const InT *in, OutT *out, VT *acc, cudaStream_t s) {
  const StreamDir &D = upper ? P.sbwd : P.sfwd;
  constexpr bool f64 = sizeof(VT) == 8;
  const VT *ext_v = reinterpret_cast<const VT *>(f64 ? (const void *)D.ext_v64.p : (const void *)D.ext_v32.p);
  const int smem_cap = 220 * 1024;
  static std::once_flag attr_once[kMaxDevices];
  once_per_device(attr_once, [&] {
    RCHOL_CUDA(cudaFuncSetAttribute(block_kernel<VT, OutT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    smem_cap));
    RCHOL_CUDA(cudaFuncSetAttribute(block_kernel<VT, OutT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    smem_cap));
    RCHOL_CUDA(cudaFuncSetAttribute(team_kernel<VT, OutT, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    smem_cap));
    RCHOL_CUDA(cudaFuncSetAttribute(team_kernel<VT, OutT, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    smem_cap));
  });
  BlockArgs<VT> a;
  a.nodes = D.nodes.p;
  a.blocks = D.blocks.p;
  a.blk_off = D.blk_off.p;
  a.acc = acc;
  a.upper = upper;
  TeamArgs<VT> ta;
  ta.nodes = D.nodes.p;
  ta.blocks = D.blocks.p;
  ta.blk_off = D.blk_off.p;
  ta.acc = acc;
  for (size_t st = 0; st + 1 < D.stage_ptr.size(); ++st) {
    const int pieces = D.stage_ptr[st + 1] - D.stage_ptr[st];
    if (!pieces) continue;
    const int64_t r0 = D.stage_row_ptr[st], r1 = D.stage_row_ptr[st + 1], nr = r1 - r0;
    const int lanes = D.stage_ext_lanes[st];
    const unsigned eg = (unsigned)((nr * lanes + 255) / 256);
    switch (lanes) {
      case 1:
        ext_kernel<VT, InT, OutT><<<eg, 256, 0, s>>>(D.srows.p + r0, nr, D.ext_rp.p, D.ext_ci.p, ext_v, in, out, acc);
        break;
      case 4:
        ext_lanes_kernel<VT, InT, OutT, 4>
            <<<eg, 256, 0, s>>>(D.srows.p + r0, nr, D.ext_rp.p, D.ext_ci.p, ext_v, in, out, acc);
        break;
      case 8:
        ext_lanes_kernel<VT, InT, OutT, 8>
            <<<eg, 256, 0, s>>>(D.srows.p + r0, nr, D.ext_rp.p, D.ext_ci.p, ext_v, in, out, acc);
        break;
      default:
        ext_lanes_kernel<VT, InT, OutT, 32>
            <<<eg, 256, 0, s>>>(D.srows.p + r0, nr, D.ext_rp.p, D.ext_ci.p, ext_v, in, out, acc);
        break;
    }
    note_launch();
    const size_t xs_bytes = (size_t)D.stage_rows[st] * sizeof(VT);
    if (D.stage_team[st]) {
      ta.node0 = D.stage_ptr[st];
      ta.bufbytes = (int)al16((size_t)D.stage_maxrec[st]);
      ta.maxchunk = D.stage_chunks[st];
      const size_t fixed = al16((size_t)ta.maxchunk * sizeof(VT)) + 2 * BS * sizeof(VT) + xs_bytes;
      // the deepest ring that fits (records arrive ring-3 steps ahead of use)
      // where few pieces share the GPU; where many do, they hide each
      // other's latency and shared memory goes to residency instead
      int ring = pieces > 2 * sm_count() ? 5 : TEAM_RING_MAX;
      while (ring > 3 && fixed + (size_t)ring * ta.bufbytes > (size_t)smem_cap) --ring;
      ta.ring = ring;
      const size_t bytes = (size_t)ring * ta.bufbytes + fixed;
      if (bytes > (size_t)smem_cap) throw Error(RCHOL_ERR_INTERNAL, "triangular-solve piece exceeds shared memory");
      const unsigned threads = 32u * (unsigned)D.stage_warps[st];
      if (upper) team_kernel<VT, OutT, true><<<pieces, threads, bytes, s>>>(ta, out);
      else team_kernel<VT, OutT, false><<<pieces, threads, bytes, s>>>(ta, out);
    } else {
      a.node0 = D.stage_ptr[st];
      a.node1 = D.stage_ptr[st + 1];
      a.bufbytes = (int)al16((size_t)D.stage_maxrec[st]);
      // deep rings for the few long chains at the top of the tree (latency),
      // shallower ones where many pieces share an SM (they hide each other)
      int nbuf = pieces >= 256 ? 4 : 6;
      while (nbuf > 2 && (size_t)nbuf * a.bufbytes + xs_bytes > (size_t)smem_cap) --nbuf;
      a.nbuf = nbuf;
      a.per_warp = (int)al16((size_t)nbuf * a.bufbytes + xs_bytes);
      int wpb = std::max(1, std::min(4, smem_cap / a.per_warp));
      if (a.per_warp > smem_cap) throw Error(RCHOL_ERR_INTERNAL, "triangular-solve piece exceeds shared memory");
      wpb = std::min(wpb, pieces);
      a.wpb = wpb;
      const int grid = (pieces + wpb - 1) / wpb;
      if (upper) block_kernel<VT, OutT, true><<<grid, 32 * wpb, (size_t)a.per_warp * wpb, s>>>(a, out);
      else block_kernel<VT, OutT, false><<<grid, 32 * wpb, (size_t)a.per_warp * wpb, s>>>(a, out);
    }
    note_launch();
    RCHOL_CUDA(cudaGetLastError());
  }
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
    ta.bufbytes = (int)al16((size_t)D.stage_maxrec[st]);
    const size_t fixed = 2 * (size_t)BS * KW * sizeof(VT) + (size_t)D.stage_rows[st] * KW * sizeof(VT);
    int ring = pieces > 2 * sm_count() ? 5 : TEAM_RING_MAX;
    while (ring > 3 && fixed + (size_t)ring * ta.bufbytes > (size_t)smem_cap) --ring;
    ta.ring = ring;
    const size_t bytes = (size_t)ring * ta.bufbytes + fixed;
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
