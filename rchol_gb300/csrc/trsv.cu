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
//                 (columns already solved); one thread per row, all SMs.
//   block_kernel  one warp per piece: the piece's unknowns live in the warp's
//                 shared memory, block records stream in through a cp.async
//                 double buffer, and per block lane r forms
//                   t_r = acc_r - sum_{earlier blocks} G_rj x_j   (sparse)
//                   x_r = sum_c (T^-1)_{rc} t_c                   (dense, 32 shuffles)
//                 no block-wide barrier anywhere.
// Values are FP32 or FP64 as the factor is stored; the block inverses are
// computed in FP64 on the host and rounded to the stored precision.

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "common.hpp"
#include "host.hpp"
#include "plan.hpp"

namespace rchol {

namespace {

constexpr int BS = 32;  // rows per block

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~size_t(15); }

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
                 o_min = o_val + al16(vsz * nent), len = o_min + al16(vsz * BS * BS);
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
    for (int c = 0; c < BS; ++c)
      for (int r = 0; r < BS; ++r) {
        const double m = (r < nr && c < nr) ? X[r][c] : 0.0;
        if (vsz == 8) std::memcpy(p + o_min + 8 * (c * BS + r), &m, 8);
        else {
          float f = (float)m;
          std::memcpy(p + o_min + 4 * (c * BS + r), &f, 4);
        }
      }
    P.offs.push_back((int64_t)P.bytes.size());
    P.maxrec = std::max<int32_t>(P.maxrec, (int32_t)len);
    P.sparse += nent;
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

// acc_i = rhs_i - sum over row i's entries outside its piece.
template <typename VT, typename InT, typename OutT>
__global__ void __launch_bounds__(256) ext_kernel(const int32_t *__restrict__ rows, int64_t nrows,
                                                  const int64_t *__restrict__ ext_rp, const int32_t *__restrict__ ext_ci,
                                                  const VT *__restrict__ ext_v, const InT *__restrict__ in,
                                                  const OutT *out, VT *__restrict__ acc) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= nrows) return;
  const int64_t i = rows[t];
  const int64_t q0 = ext_rp[i], q1 = ext_rp[i + 1];
  VT s0 = 0, s1 = 0;
  int64_t q = q0;
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
  int per_warp;         // shared-memory bytes per warp
  const unsigned char *blocks;
  const int64_t *blk_off;
  const VT *acc;
};

template <typename VT, typename OutT>
__global__ void __launch_bounds__(128) block_kernel(BlockArgs<VT> a, OutT *out) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int piece = a.node0 + blockIdx.x * a.wpb + w;
  if (piece >= a.node1) return;  // the whole warp leaves
  const NodeDesc nd = a.nodes[piece];
  unsigned char *base = smem + (size_t)w * a.per_warp;
  unsigned char *buf0 = base, *buf1 = base + a.bufbytes;
  VT *xs = reinterpret_cast<VT *>(base + 2 * (size_t)a.bufbytes);
  const unsigned char *src = a.blocks;
  const int64_t *boff = a.blk_off + nd.blk0;

  auto load = [&](int k, unsigned char *dst) {
    const int64_t o0 = boff[k], len = boff[k + 1] - o0;
    for (int64_t o = lane * 16; o < len; o += 32 * 16) cp_async16(dst + o, src + o0 + o);
    cp_async_commit();
  };
  if (nd.nblocks > 0) load(0, buf0);
  if (nd.nblocks > 1) load(1, buf1);
  for (int r = lane; r < nd.rows; r += 32) xs[r] = a.acc[nd.begin + r];
  __syncwarp();

  for (int k = 0; k < nd.nblocks; ++k) {
    if (k + 1 < nd.nblocks) cp_async_wait<1>();
    else cp_async_wait<0>();
    __syncwarp();
    const unsigned char *p = (k & 1) ? buf1 : buf0;
    const uint32_t *hdr = reinterpret_cast<const uint32_t *>(p);
    const uint32_t nr = hdr[0], nent = hdr[1], row0 = hdr[2], csz = hdr[3];
    const uint32_t *eoff = reinterpret_cast<const uint32_t *>(p + 16);
    const size_t o_col = 16 + al16(4 * (BS + 1));
    const size_t o_val = o_col + al16((size_t)csz * nent);
    const size_t o_min = o_val + al16(sizeof(VT) * nent);
    const VT *val = reinterpret_cast<const VT *>(p + o_val);
    const VT *minv = reinterpret_cast<const VT *>(p + o_min);
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
    VT c0 = 0, c1 = 0, c2 = 0, c3 = 0;
#pragma unroll
    for (int c = 0; c < BS; c += 4) {
      c0 += minv[(c + 0) * BS + lane] * __shfl_sync(0xffffffffu, t, c + 0);
      c1 += minv[(c + 1) * BS + lane] * __shfl_sync(0xffffffffu, t, c + 1);
      c2 += minv[(c + 2) * BS + lane] * __shfl_sync(0xffffffffu, t, c + 2);
      c3 += minv[(c + 3) * BS + lane] * __shfl_sync(0xffffffffu, t, c + 3);
    }
    if (lane < (int)nr) xs[row0 + lane] = (c0 + c1) + (c2 + c3);
    __syncwarp();
    if (k + 2 < nd.nblocks) load(k + 2, (k & 1) ? buf1 : buf0);
  }
  __syncwarp();
  for (int r = lane; r < nd.rows; r += 32) out[nd.begin + r] = (OutT)xs[r];
}

}  // namespace

// ---- plan construction ---------------------------------------------------------------

// Host copy of one direction's stream (development checks decode it on the CPU).
struct HostStreamCopy {
  std::vector<unsigned char> blocks;
  std::vector<int64_t> blk_off;
  std::vector<NodeDesc> desc;
  std::vector<int64_t> ext_rp;
  std::vector<int32_t> ext_ci;
  std::vector<double> ext_v;
  std::vector<int> stage_ptr;
};

static void build_dir_streams(const std::vector<int64_t> &rp, const std::vector<int32_t> &ci,
                              const std::vector<double> &v, int64_t n, const std::vector<TreeNode> &tnodes,
                              bool upper, bool fp32, StreamDir &D, cudaStream_t s,
                              HostStreamCopy *host_copy = nullptr) {
  const size_t vsz = fp32 ? 4 : 8;
  // Pieces: a node is cut into consecutive pieces (whole blocks) so that one
  // warp's shared memory holds the piece's unknowns plus two block buffers.
  // The bound of a block record counts every entry of its rows that lies in
  // the node but outside the block (an upper bound of its sparse part).
  const size_t budget = 200 * 1024;
  int maxdepth = 1;
  for (auto &nd : tnodes) maxdepth = std::max(maxdepth, nd.depth);
  struct Piece {
    int64_t b, e;
  };
  auto cut_node = [&](int64_t b, int64_t e) {
    std::vector<Piece> out;
    const int64_t nb = (e - b + BS - 1) / BS;
    std::vector<size_t> recb(nb);
    parallel_for(nb, [&](int64_t k0, int64_t k1) {
      for (int64_t k = k0; k < k1; ++k) {
        const int64_t r0 = b + k * BS, r1 = std::min(e, r0 + BS);
        size_t cnt = 0;
        for (int64_t i = r0; i < r1; ++i)
          for (int64_t q = rp[i]; q < rp[i + 1]; ++q) cnt += (ci[q] >= b && ci[q] < e && (ci[q] < r0 || ci[q] >= r1));
        recb[k] = 16 + al16(4 * (BS + 1)) + al16(4 * cnt) + al16(vsz * cnt) + al16(vsz * BS * BS);
      }
    }, 256);
    int64_t k = 0;
    while (k < nb) {
      int64_t k1 = k;
      size_t mx = 0;
      while (k1 < nb) {
        const size_t m2 = std::max(mx, recb[k1]);
        const int64_t rows = std::min(e, b + (k1 + 1) * BS) - (b + k * BS);
        if (k1 > k && (2 * al16(m2) + (size_t)rows * vsz > budget || rows > 65535)) break;
        mx = m2;
        ++k1;
      }
      if (2 * al16(mx) + (size_t)(std::min(e, b + k1 * BS) - (b + k * BS)) * vsz > budget)
        throw Error(RCHOL_ERR_INTERNAL, "a 32-row block of G is too dense for the shared-memory solve");
      out.push_back(Piece{b + k * BS, std::min(e, b + k1 * BS)});
      k = k1;
    }
    return out;
  };
  std::vector<Piece> pieces;
  D.stage_ptr.assign(1, 0);
  for (int st = 0; st < maxdepth; ++st) {
    const int depth = upper ? st + 1 : maxdepth - st;
    std::vector<std::vector<Piece>> by_index;  // piece j of every node of this depth
    for (auto &nd : tnodes) {
      if (nd.depth != depth) continue;
      const int64_t b = nd.begin, e = std::min(nd.end, n);
      if (e <= b) continue;
      std::vector<Piece> ps = cut_node(b, e);
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
  // block records
  std::vector<PieceBuild> built(np);
  parallel_for(np, [&](int64_t k0, int64_t k1) {
    for (int64_t k = k0; k < k1; ++k) build_piece(rp, ci, v, pieces[k].b, pieces[k].e, upper, vsz, built[k]);
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
  D.stage_split.clear();
  D.stage_rows.clear();
  D.stage_maxrec.clear();
  D.stage_row_ptr.assign(1, 0);
  D.steps = 0;
  std::vector<int32_t> srows;
  for (size_t st = 0; st + 1 < D.stage_ptr.size(); ++st) {
    int rows = 0, maxrec = 16, steps = 0;
    for (int k = D.stage_ptr[st]; k < D.stage_ptr[st + 1]; ++k) {
      rows = std::max(rows, desc[k].rows);
      maxrec = std::max(maxrec, desc[k].maxrec);
      steps = std::max(steps, desc[k].nblocks);
      for (int64_t i = desc[k].begin; i < desc[k].begin + desc[k].rows; ++i) srows.push_back((int32_t)i);
    }
    D.stage_split.push_back(1);
    D.stage_rows.push_back(rows);
    D.stage_maxrec.push_back(maxrec);
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

void build_streams(const rchol_factor_s &F, SolvePlan &P, cudaStream_t s) {
  const int64_t n = F.n, nnz = F.nnz;
  const bool fp32 = F.precision == RCHOL_PREC_FP32;
  std::vector<int64_t> rp(n + 1);
  std::vector<int32_t> ci(nnz);
  std::vector<double> v(nnz);
  F.lrp.download(rp.data(), n + 1, s);
  F.lci.download(ci.data(), nnz, s);
  F.lv.download(v.data(), nnz, s);
  RCHOL_CUDA(cudaStreamSynchronize(s));
  build_dir_streams(rp, ci, v, n, F.nodes, false, fp32, P.sfwd, s);
  F.urp.download(rp.data(), n + 1, s);
  F.uci.download(ci.data(), nnz, s);
  F.uv.download(v.data(), nnz, s);
  RCHOL_CUDA(cudaStreamSynchronize(s));
  build_dir_streams(rp, ci, v, n, F.nodes, true, fp32, P.sbwd, s);
}

// ---- launch ------------------------------------------------------------------------------

template <typename VT, typename InT, typename OutT>
static void launch_streams(const SolvePlan &P, bool upper, const InT *in, OutT *out, VT *acc, cudaStream_t s) {
  const StreamDir &D = upper ? P.sbwd : P.sfwd;
  constexpr bool f64 = sizeof(VT) == 8;
  const VT *ext_v = reinterpret_cast<const VT *>(f64 ? (const void *)D.ext_v64.p : (const void *)D.ext_v32.p);
  const int smem_cap = 220 * 1024;
  static bool attr = false;
  if (!attr) {
    RCHOL_CUDA(cudaFuncSetAttribute(block_kernel<VT, OutT>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_cap));
    attr = true;
  }
  BlockArgs<VT> a;
  a.nodes = D.nodes.p;
  a.blocks = D.blocks.p;
  a.blk_off = D.blk_off.p;
  a.acc = acc;
  for (size_t st = 0; st + 1 < D.stage_ptr.size(); ++st) {
    const int pieces = D.stage_ptr[st + 1] - D.stage_ptr[st];
    if (!pieces) continue;
    const int64_t r0 = D.stage_row_ptr[st], r1 = D.stage_row_ptr[st + 1];
    ext_kernel<VT, InT, OutT><<<(unsigned)((r1 - r0 + 255) / 256), 256, 0, s>>>(
        D.srows.p + r0, r1 - r0, D.ext_rp.p, D.ext_ci.p, ext_v, in, out, acc);
    note_launch();
    a.node0 = D.stage_ptr[st];
    a.node1 = D.stage_ptr[st + 1];
    a.bufbytes = (int)al16((size_t)D.stage_maxrec[st]);
    a.per_warp = (int)al16(2 * (size_t)a.bufbytes + (size_t)D.stage_rows[st] * sizeof(VT));
    int wpb = std::max(1, std::min(4, smem_cap / a.per_warp));
    if (a.per_warp > smem_cap) throw Error(RCHOL_ERR_INTERNAL, "triangular-solve piece exceeds shared memory");
    wpb = std::min(wpb, pieces);
    a.wpb = wpb;
    const int grid = (pieces + wpb - 1) / wpb;
    block_kernel<VT, OutT><<<grid, 32 * wpb, (size_t)a.per_warp * wpb, s>>>(a, out);
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

}  // namespace rchol
