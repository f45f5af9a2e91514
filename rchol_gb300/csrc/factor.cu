// Randomized Cholesky factorization of the extended Laplacian on the GPU.
//
// Replaces c++/rchol_lap/rchol_lap.cpp: process_array (:778-855),
// recursive_calculation (:187-355), linear_update (:733-770),
// random_sampling0 (:643-729) and coalesce (:358-387).
//
// Schedule.  The nested-dissection tree is processed one depth at a time,
// leaves first.  One warp owns one tree node and eliminates its columns in
// order; nodes of the same depth are independent (a fill edge never joins two
// sibling subtrees), so a launch covers every node of a depth.
//
// Column store.  Every column c owns a slab of fill records {row, source, w}
// in HBM (capacity fcap[c]).  Eliminating column j appends each sampled edge
// to the slab of its smaller endpoint with one atomicAdd on that column's
// counter -- the same store serves node-internal fill (the reference's
// gsl_spmatrix_set) and fill deferred to an ancestor separator (its sep_edge
// lists).  A slab that would overflow sets a flag; the host then enlarges the
// slabs that overflowed and runs the factorization again, which gives the
// same result because nothing depends on timing.
//
// Per column (one warp, shared memory only):
//   1. gather the initial entries (CSR row c of the upper extended Laplacian,
//      minus the diagonal and negative ground edges) and the fill records;
//   2. sort by (row, source) and sum duplicate rows left to right;
//   3. sort by (weight, row), prefix sum in 32-wide Hillis-Steele chunks;
//      (sorts: ranks in one pass over the keys up to 128 records, a bitonic
//      network past that; the keys are unique, so both give one order)
//   4. sample the m-1 fill edges in parallel, one lane per edge, with a
//      Philox4x32-10 uniform keyed by (seed, c, i) and a binary search;
//   5. write the column of G: sqrt(d) then -(w/d)*sqrt(d) per row.
// All rounding is explicit (_rn intrinsics), so the result equals the
// device-contract mode of the CPU restatement bit for bit.

#include <algorithm>
#include <cstring>
#include <vector>

#include "common.hpp"
#include "host.hpp"

namespace rchol {

namespace {

struct FillRec {
  uint32_t row;
  uint32_t src;  // eliminated column + 1
  double w;
};
static_assert(sizeof(FillRec) == 16, "FillRec layout");

enum { FLAG_FILL = 0, FLAG_WIDTH = 1, FLAG_GCAP = 2, FLAG_SINGULAR = 3, NFLAGS = 4 };

struct ElimArgs {
  const int64_t *lrp;  // extended Laplacian, upper CSR
  const int32_t *lci;
  const double *lv;
  int64_t lnnz;        // entries of lci / lv
  int64_t next;        // n + 1 (ground vertex = next - 1)
  const int64_t *node_begin;
  const int64_t *node_end;
  int num_nodes;
  uint32_t *fcnt;
  const uint32_t *fcap;
  const int64_t *fbase;
  FillRec *frec;
  int64_t *gstart;
  uint32_t *gcnt;
  int32_t *grow;
  double *gval;
  unsigned long long *gtop;
  int64_t gcap;
  double *diag;
  int *flags;
  uint64_t seed;
  int emax;                  // per-warp buffer capacity in entries
  unsigned char *gscratch;   // per-warp buffers in HBM when they exceed shared memory
};

__device__ __forceinline__ uint32_t mulhi32(uint32_t a, uint32_t b) { return __umulhi(a, b); }

// Philox4x32-10 (Salmon et al., SC'11).
__device__ __forceinline__ void philox(uint32_t c[4], uint32_t k0, uint32_t k1) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += 0x9E3779B9u;
      k1 += 0xBB67AE85u;
    }
    uint32_t hi0 = mulhi32(0xD2511F53u, c[0]), lo0 = 0xD2511F53u * c[0];
    uint32_t hi1 = mulhi32(0xCD9E8D57u, c[2]), lo1 = 0xCD9E8D57u * c[2];
    uint32_t n0 = hi1 ^ c[1] ^ k0, n2 = hi0 ^ c[3] ^ k1;
    c[0] = n0;
    c[1] = lo1;
    c[2] = n2;
    c[3] = lo0;
  }
}

__device__ __forceinline__ double uniform53(uint64_t seed, uint64_t v, uint32_t i) {
  uint32_t c[4] = {i >> 1, 0u, (uint32_t)v, (uint32_t)(v >> 32)};
  philox(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  uint32_t a = (i & 1) ? c[2] : c[0];
  uint32_t b = (i & 1) ? c[3] : c[1];
  return __dmul_rn(__dadd_rn(__dmul_rn((double)(a >> 5), 67108864.0), (double)(b >> 6)),
                   1.0 / 9007199254740992.0);
}

__device__ __forceinline__ bool wless(double wa, uint32_t ra, double wb, uint32_t rb) {
  return wa < wb || (wa == wb && ra < rb);
}

// A double as an unsigned integer with the same order (negative zero taken
// as zero, so equal weights stay equal): compares then run on the integer
// pipes, which GB300 has many more of than FP64 ones.
__device__ __forceinline__ uint64_t wkey(double w) {
  uint64_t b = (uint64_t)__double_as_longlong(w);
  if (b == 0x8000000000000000ull) b = 0;
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

constexpr unsigned GCHUNK = 256;  // entries of G a warp reserves at a time

// In-place ascending sort of n records (key[i], val[i]) by one warp: a
// bitonic network whose merges compare each element with its mirror, so
// every comparator points the same way and the missing elements past n
// behave as +infinity (comparators reaching past n are skipped).  O(n log^2 n)
// work against the O(n^2) of a rank sort; used for wide columns.  The keys of
// a column are unique, so the order equals any other sort's.
template <typename K, typename V, typename Less>
__device__ void warp_bitonic_sort(K *key, V *val, int n, Less less) {
  const int lane = threadIdx.x & 31;
  int npow = 1;
  while (npow < n) npow <<= 1;
  const int half = npow >> 1;
  int lk = 1;  // log2(k)
  for (int k = 2; k <= npow; k <<= 1, ++lk) {
    const int hk = k >> 1;
    for (int t = lane; t < half; t += 32) {  // mirror stage
      const int blk = t >> (lk - 1), o = t & (hk - 1);
      const int i = (blk << lk) + o, j = (blk << lk) + k - 1 - o;
      if (j < n && less(key[j], val[j], key[i], val[i])) {
        const K tk = key[i];
        key[i] = key[j];
        key[j] = tk;
        const V tv = val[i];
        val[i] = val[j];
        val[j] = tv;
      }
    }
    __syncwarp();
    for (int ld = lk - 2; ld >= 0; --ld) {  // half cleaners, distance d = 2^ld
      const int d = 1 << ld;
      for (int t = lane; t < half; t += 32) {
        const int i = ((t >> ld) << (ld + 1)) + (t & (d - 1)), j = i + d;
        if (j < n && less(key[j], val[j], key[i], val[i])) {
          const K tk = key[i];
          key[i] = key[j];
          key[j] = tk;
          const V tv = val[i];
          val[i] = val[j];
          val[j] = tv;
        }
      }
      __syncwarp();
    }
  }
}

// Rank sorts of up to 32 * PER records with unique keys: lane l owns records
// l, l + 32, ..., and one pass over all keys (four loads in flight) counts,
// for each of them, the keys that order before it; the record then moves to
// its rank.  Keys: (row << 32 | source) for the merge order, (weight as
// order-preserving bits, row) for the sampling order.
template <int PER>
__device__ __forceinline__ void rank_sort_rowsrc(const uint64_t *key, const double *val, int n, uint64_t *okey,
                                                 double *oval, int lane) {
  uint64_t mine[PER];
  int rank[PER];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int e = lane + 32 * p;
    mine[p] = e < n ? key[e] : 0;
    rank[p] = 0;
  }
  int f = 0;
  for (; f + 4 <= n; f += 4) {
    const uint64_t k0 = key[f], k1 = key[f + 1], k2 = key[f + 2], k3 = key[f + 3];
#pragma unroll
    for (int p = 0; p < PER; ++p)
      rank[p] += (int)(k0 < mine[p]) + (int)(k1 < mine[p]) + (int)(k2 < mine[p]) + (int)(k3 < mine[p]);
  }
  for (; f < n; ++f) {
    const uint64_t k0 = key[f];
#pragma unroll
    for (int p = 0; p < PER; ++p) rank[p] += (int)(k0 < mine[p]);
  }
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int e = lane + 32 * p;
    if (e < n) {
      okey[rank[p]] = mine[p];
      oval[rank[p]] = val[e];
    }
  }
}

// wk: order-preserving weight bits; rows in the low 32 bits of row.
template <int PER>
__device__ __forceinline__ void rank_sort_weight(const uint64_t *wk, const uint64_t *row, const double *val, int n,
                                                 uint64_t *orow, double *oval, int lane) {
  uint64_t mw[PER];
  uint32_t mr[PER];
  int rank[PER];
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int e = lane + 32 * p;
    mw[p] = e < n ? wk[e] : 0;
    mr[p] = e < n ? (uint32_t)row[e] : 0;
    rank[p] = 0;
  }
  auto before = [](uint64_t wf, uint32_t rf, uint64_t we, uint32_t re) {
    return (int)((wf < we) | ((wf == we) & (rf < re)));
  };
  int f = 0;
  for (; f + 4 <= n; f += 4) {
    const uint64_t w0 = wk[f], w1 = wk[f + 1], w2 = wk[f + 2], w3 = wk[f + 3];
    const uint32_t r0 = (uint32_t)row[f], r1 = (uint32_t)row[f + 1], r2 = (uint32_t)row[f + 2],
                   r3 = (uint32_t)row[f + 3];
#pragma unroll
    for (int p = 0; p < PER; ++p)
      rank[p] += before(w0, r0, mw[p], mr[p]) + before(w1, r1, mw[p], mr[p]) + before(w2, r2, mw[p], mr[p]) +
                 before(w3, r3, mw[p], mr[p]);
  }
  for (; f < n; ++f) {
    const uint64_t w0 = wk[f];
    const uint32_t r0 = (uint32_t)row[f];
#pragma unroll
    for (int p = 0; p < PER; ++p) rank[p] += before(w0, r0, mw[p], mr[p]);
  }
#pragma unroll
  for (int p = 0; p < PER; ++p) {
    const int e = lane + 32 * p;
    if (e < n) {
      orow[rank[p]] = mr[p];
      oval[rank[p]] = val[e];
    }
  }
}

constexpr int RANK_SORT_MAX = 128;  // wider columns use the bitonic network

__global__ void eliminate_kernel(ElimArgs a) {
  extern __shared__ unsigned char smem_raw[];
  const int lane = threadIdx.x & 31;
  const int wib = threadIdx.x >> 5;
  const int warp = blockIdx.x * (blockDim.x >> 5) + wib;
  if (warp >= a.num_nodes) return;
  const int E = a.emax;
  // per-warp layout: akey[E] aval[E] bkey[E] bval[E] cs[E]
  unsigned char *base = a.gscratch ? a.gscratch + (size_t)warp * (size_t)E * 40
                                   : smem_raw + (size_t)wib * (size_t)E * 40;
  uint64_t *akey = reinterpret_cast<uint64_t *>(base);
  double *aval = reinterpret_cast<double *>(base + (size_t)E * 8);
  uint64_t *bkey = reinterpret_cast<uint64_t *>(base + (size_t)E * 16);
  double *bval = reinterpret_cast<double *>(base + (size_t)E * 24);
  double *cs = reinterpret_cast<double *>(base + (size_t)E * 32);

  const int64_t ground = a.next - 1;
  const int64_t cb = a.node_begin[warp], ce = a.node_end[warp];
  // The next column's static inputs (row range, fill slab, first 32 initial
  // entries) are loaded one column ahead, so their latency overlaps the
  // current column; only its fill count and records wait for the current one.
  int64_t nx_r1 = a.lrp[cb], nx_r2 = a.lrp[cb + 1];
  uint32_t nx_cap = a.fcap[cb];
  int64_t nx_fb = a.fbase[cb];
  int32_t nx_col = 0;
  double nx_v = 0.0;
  if (nx_r1 + lane < nx_r2) {
    nx_col = a.lci[nx_r1 + lane];
    nx_v = a.lv[nx_r1 + lane];
  }
  unsigned long long gcur = 0, gend = 0;  // lane 0: this warp's reserved run of G
  for (int64_t c = cb; c < ce; ++c) {
    // ---- 1. gather ----------------------------------------------------------
    const int64_t r0 = nx_r1, r1 = nx_r2;
    const uint32_t cap = nx_cap;
    const int64_t fb = nx_fb;
    const int32_t pre_col = nx_col;
    const double pre_v = nx_v;
    if (c + 1 < ce) {  // rows of column c+1 start at r1; lci/lv reads stay inside the arrays
      nx_r1 = r1;
      nx_r2 = a.lrp[c + 2];
      nx_cap = a.fcap[c + 1];
      nx_fb = a.fbase[c + 1];
      if (r1 + lane < a.lnnz) {
        nx_col = a.lci[r1 + lane];
        nx_v = a.lv[r1 + lane];
      }
    }
    uint32_t nfill = __ldcg(&a.fcnt[c]);
    if (nfill > cap) nfill = cap;  // overflow already flagged by the writer
    int ninit = 0;
    // initial entries: count kept ones with a ballot per 32-wide chunk
    for (int64_t k0 = r0; k0 < r1; k0 += 32) {
      int64_t k = k0 + lane;
      bool keep = false;
      int32_t col = 0;
      double v = 0.0;
      if (k < r1) {
        col = k0 == r0 ? pre_col : a.lci[k];
        v = k0 == r0 ? pre_v : a.lv[k];
        keep = (col != c) && !(col == ground && v < 0.0 && c != ground);
      }
      unsigned bal = __ballot_sync(0xffffffffu, keep);
      int pos = ninit + __popc(bal & ((1u << lane) - 1u));
      if (keep && pos < E) {
        akey[pos] = ((uint64_t)(uint32_t)col << 32);
        aval[pos] = v;
      }
      ninit += __popc(bal);
    }
    int total = ninit + (int)nfill;
    if (total > E) {
      if (lane == 0) atomicMax(&a.flags[FLAG_WIDTH], total);
      total = 0;  // skip the column; the host retries with wider buffers
    }
    // fill records: one 16-byte load each, two per lane in flight
    for (uint32_t f0 = lane; f0 < nfill && total; f0 += 64) {
      const uint32_t f1 = f0 + 32;
      const uint4 q0 = __ldcg(reinterpret_cast<const uint4 *>(a.frec + fb + f0));
      uint4 q1 = make_uint4(0u, 0u, 0u, 0u);
      if (f1 < nfill) q1 = __ldcg(reinterpret_cast<const uint4 *>(a.frec + fb + f1));
      akey[ninit + f0] = ((uint64_t)q0.x << 32) | q0.y;  // {row, src, w}
      aval[ninit + f0] = __hiloint2double((int)q0.w, (int)q0.z);
      if (f1 < nfill) {
        akey[ninit + f1] = ((uint64_t)q1.x << 32) | q1.y;
        aval[ninit + f1] = __hiloint2double((int)q1.w, (int)q1.z);
      }
    }
    __syncwarp();
    // ---- 2. sort by (row, source) and merge --------------------------------
    if (total <= 32) {
      rank_sort_rowsrc<1>(akey, aval, total, bkey, bval, lane);
    } else if (total <= 64) {
      rank_sort_rowsrc<2>(akey, aval, total, bkey, bval, lane);
    } else if (total <= RANK_SORT_MAX) {
      rank_sort_rowsrc<4>(akey, aval, total, bkey, bval, lane);
    } else {
      warp_bitonic_sort(akey, aval, total,
                        [](uint64_t ka, double, uint64_t kb, double) { return ka < kb; });
      for (int e = lane; e < total; e += 32) {
        bkey[e] = akey[e];
        bval[e] = aval[e];
      }
    }
    __syncwarp();
    // Records e and e + 32 of a lane are merged together: the first record
    // of each row (its head) sums the row's duplicates left to right, both
    // heads' runs in one loop.
    int m = 0;
    auto row_of = [&](int e) { return (uint32_t)(bkey[e] >> 32); };
    for (int e0 = 0; e0 < total; e0 += 64) {
      const int ea = e0 + lane, eb = ea + 32;
      bool ha = false, hb = false;
      uint32_t rowa = 0, rowb = 0;
      if (ea < total) {
        rowa = row_of(ea);
        ha = (ea == 0) || (row_of(ea - 1) != rowa);
      }
      if (eb < total) {
        rowb = row_of(eb);
        hb = row_of(eb - 1) != rowb;
      }
      double sa = ha ? bval[ea] : 0.0, sb = hb ? bval[eb] : 0.0;
      int fa = ea + 1, fb = eb + 1;
      bool ga = ha, gb = hb;
      while (ga || gb) {
        if (ga) {
          if (fa < total && row_of(fa) == rowa) sa = __dadd_rn(sa, bval[fa++]);
          else ga = false;
        }
        if (gb) {
          if (fb < total && row_of(fb) == rowb) sb = __dadd_rn(sb, bval[fb++]);
          else gb = false;
        }
      }
      const unsigned lt = (1u << lane) - 1u;
      const unsigned bala = __ballot_sync(0xffffffffu, ha), balb = __ballot_sync(0xffffffffu, hb);
      const int pa = m + __popc(bala & lt), pb = m + __popc(bala) + __popc(balb & lt);
      if (ha) {
        akey[pa] = rowa;  // rows ascending
        aval[pa] = sa;
      }
      if (hb) {
        akey[pb] = rowb;
        aval[pb] = sb;
      }
      m += __popc(bala) + __popc(balb);
    }
    __syncwarp();
    // ---- 3. sort by (weight, row), prefix sum --------------------------------
    if (m <= RANK_SORT_MAX) {
      uint64_t *wk = reinterpret_cast<uint64_t *>(cs);  // cs is free until the prefix sum
      for (int e = lane; e < m; e += 32) wk[e] = wkey(aval[e]);
      __syncwarp();
      if (m <= 32) rank_sort_weight<1>(wk, akey, aval, m, bkey, bval, lane);
      else if (m <= 64) rank_sort_weight<2>(wk, akey, aval, m, bkey, bval, lane);
      else rank_sort_weight<4>(wk, akey, aval, m, bkey, bval, lane);
      __syncwarp();  // every lane's reads of wk end before the prefix sum reuses cs
    } else {
      for (int e = lane; e < m; e += 32) {
        bkey[e] = (uint32_t)akey[e];
        bval[e] = aval[e];
      }
      __syncwarp();
      warp_bitonic_sort(bkey, bval, m,
                        [](uint64_t ra, double wa, uint64_t rb, double wb) {
                          return wless(wa, (uint32_t)ra, wb, (uint32_t)rb);
                        });
    }
    __syncwarp();
    // inclusive prefix sum in 32-wide chunks (Hillis-Steele inside a chunk,
    // then the running carry), two chunks scanned side by side
    double carry = 0.0;
    for (int e0 = 0; e0 < m; e0 += 64) {
      const int ea = e0 + lane, eb = ea + 32;
      double va = (ea < m) ? bval[ea] : 0.0, vb = (eb < m) ? bval[eb] : 0.0;
#pragma unroll
      for (int d = 1; d < 32; d <<= 1) {
        const double ta = __shfl_up_sync(0xffffffffu, va, d), tb = __shfl_up_sync(0xffffffffu, vb, d);
        if (lane >= d) {
          va = __dadd_rn(ta, va);
          vb = __dadd_rn(tb, vb);
        }
      }
      const double outa = __dadd_rn(carry, va);
      if (ea < m) cs[ea] = outa;
      const double ca = __shfl_sync(0xffffffffu, outa, min(31, m - 1 - e0));
      const double outb = __dadd_rn(ca, vb);
      if (eb < m) cs[eb] = outb;
      carry = __shfl_sync(0xffffffffu, outb, min(31, max(0, m - 1 - e0 - 32)));
    }
    __syncwarp();
    const double csum = m ? cs[m - 1] : 0.0;
    // ---- 4. sample ----------------------------------------------------------
    // Edges i and i + 32 of a lane are drawn together (straight-line code,
    // one search loop for both), so their latency chains overlap; the binary
    // searches compare prefix sums as order-preserving integers.
    for (int i0 = lane; i0 < m - 1; i0 += 64) {
      const bool two = i0 + 32 < m - 1;
      const int i1 = two ? i0 + 32 : i0;
      const double u0 = uniform53(a.seed, (uint64_t)c, (uint32_t)i0);
      const double u1 = uniform53(a.seed, (uint64_t)c, (uint32_t)i1);
      const double tar0 = cs[i0], tar1 = cs[i1];
      const double span0 = __dsub_rn(csum, tar0), span1 = __dsub_rn(csum, tar1);
      const uint64_t r0 = wkey(__dadd_rn(__dmul_rn(u0, span0), tar0));
      const uint64_t r1 = wkey(__dadd_rn(__dmul_rn(u1, span1), tar1));
      int lo0 = i0, hi0 = m, lo1 = i1, hi1 = m;
      while (lo0 < hi0 || lo1 < hi1) {
        const int mid0 = (lo0 + hi0) >> 1, mid1 = (lo1 + hi1) >> 1;
        const bool go0 = lo0 < hi0, go1 = lo1 < hi1;
        const uint64_t c0 = wkey(cs[go0 ? mid0 : 0]), c1 = wkey(cs[go1 ? mid1 : 0]);
        if (go0) {
          if (c0 < r0) lo0 = mid0 + 1;
          else hi0 = mid0;
        }
        if (go1) {
          if (c1 < r1) lo1 = mid1 + 1;
          else hi1 = mid1;
        }
      }
      const int k0 = lo0 < m ? lo0 : m - 1, k1 = lo1 < m ? lo1 : m - 1;
      const bool e0 = k0 != i0, e1 = two && k1 != i1;
      const double w0 = __ddiv_rn(__dmul_rn(bval[i0], span0), csum);
      const double w1 = __ddiv_rn(__dmul_rn(bval[i1], span1), csum);
      const uint32_t ri0 = (uint32_t)bkey[i0], rk0 = (uint32_t)bkey[k0];
      const uint32_t ri1 = (uint32_t)bkey[i1], rk1 = (uint32_t)bkey[k1];
      const uint32_t t0 = min(ri0, rk0), x0 = max(ri0, rk0), t1 = min(ri1, rk1), x1 = max(ri1, rk1);
      const uint32_t s0 = e0 ? atomicAdd(&a.fcnt[t0], 1u) : 0u;
      const uint32_t s1 = e1 ? atomicAdd(&a.fcnt[t1], 1u) : 0u;
      if (e0) {
        if (s0 < a.fcap[t0]) a.frec[a.fbase[t0] + s0] = FillRec{x0, (uint32_t)c + 1u, w0};
        else atomicOr(&a.flags[FLAG_FILL], 1);
      }
      if (e1) {
        if (s1 < a.fcap[t1]) a.frec[a.fbase[t1] + s1] = FillRec{x1, (uint32_t)c + 1u, w1};
        else atomicOr(&a.flags[FLAG_FILL], 1);
      }
    }
    // ---- 5. column of G -------------------------------------------------------
    if (c != ground) {
      bool hasg = (m > 0) && ((int64_t)(uint32_t)akey[m - 1] == ground);
      int cnt = 1 + m - (hasg ? 1 : 0);
      unsigned long long gs = 0;
      if (lane == 0) {
        if (gcur + (unsigned)cnt > gend) {
          const unsigned long long take = max((unsigned)cnt, GCHUNK);
          gcur = atomicAdd(a.gtop, take);
          gend = gcur + take;
        }
        gs = gcur;
        gcur += (unsigned)cnt;
        a.diag[c] = csum;
        if (!(csum > 0.0)) atomicOr(&a.flags[FLAG_SINGULAR], 1);
      }
      gs = __shfl_sync(0xffffffffu, gs, 0);
      if ((int64_t)(gs + cnt) > a.gcap) {
        if (lane == 0) atomicOr(&a.flags[FLAG_GCAP], 1);
      } else {
        double sq = __dsqrt_rn(csum);
        double inv = __ddiv_rn(1.0, csum);
        if (lane == 0) {
          a.gstart[c] = (int64_t)gs;
          a.gcnt[c] = (uint32_t)cnt;
          a.grow[gs] = (int32_t)c;
          a.gval[gs] = sq;
        }
        for (int e = lane; e < cnt - 1; e += 32) {
          a.grow[gs + 1 + e] = (int32_t)(uint32_t)akey[e];
          a.gval[gs + 1 + e] = __dmul_rn(-__dmul_rn(aval[e], inv), sq);
        }
      }
    } else if (lane == 0) {
      a.diag[c] = csum;
    }
    __syncwarp();
  }
}

// ---- CSR assembly ----------------------------------------------------------

__global__ void copy_columns_kernel(int64_t n, const int64_t *gstart, const uint32_t *gcnt,
                                    const int32_t *grow, const double *gval, const int64_t *urp,
                                    int32_t *uci, double *uv) {
  int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (warp >= n) return;
  int64_t s = gstart[warp], o = urp[warp];
  uint32_t c = gcnt[warp];
  for (uint32_t e = lane; e < c; e += 32) {
    uci[o + e] = grow[s + e];
    uv[o + e] = gval[s + e];
  }
}

__global__ void u32_to_i64_kernel(int64_t n, const uint32_t *a, int64_t *b) {
  int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}

}  // namespace

// Exclusive scan of int64 counts in place: out[0..n] with out[n] = total.
void exclusive_scan_i64(int64_t *d_data, int64_t n, cudaStream_t s);

namespace {

int pow2_at_least(int x) {
  int p = 32;
  while (p < x) p <<= 1;
  return p;
}

}  // namespace

void gpu_factor(const HostCsr &ext, const std::vector<TreeNode> &nodes, uint64_t seed,
                rchol_factor_s &F, cudaStream_t s) {
  const int64_t next = ext.n, n = next - 1;
  RCHOL_CHECK_ARG(next < (int64_t)UINT32_MAX - 1, "matrix too large for 32-bit vertex ids");
  // device copy of the extended Laplacian (int32 column indices)
  DevBuf<int64_t> lrp;
  DevBuf<int32_t> lci;
  DevBuf<double> lv;
  {
    std::vector<int32_t> ci32(ext.ci.size());
    parallel_for((int64_t)ext.ci.size(), [&](int64_t a0, int64_t b0) {
      for (int64_t i = a0; i < b0; ++i) ci32[i] = (int32_t)ext.ci[i];
    }, 1 << 20);
    lrp.upload(ext.rp.data(), ext.rp.size(), s);
    lci.upload(ci32.data(), ci32.size(), s);
    lv.upload(ext.v.data(), ext.v.size(), s);
    RCHOL_CUDA(cudaStreamSynchronize(s));
  }
  // depth of every column and node lists per depth
  int maxdepth = 1;
  for (auto &nd : nodes) maxdepth = std::max(maxdepth, nd.depth);
  std::vector<int> coldepth(next, 1);
  std::vector<char> colleaf(next, 0);
  std::vector<int32_t> colnode(next, -1);
  for (size_t j = 0; j < nodes.size(); ++j)
    for (int64_t c = nodes[j].begin; c < nodes[j].end; ++c) {
      coldepth[c] = nodes[j].depth;
      colleaf[c] = nodes[j].leaf;
      colnode[c] = (int32_t)j;
    }
  std::vector<int> initdeg(next);
  for (int64_t c = 0; c < next; ++c) initdeg[c] = (int)(ext.rp[c + 1] - ext.rp[c]);
  // initial slab capacities: small for leaf columns; separators receive the
  // deferred fill of their whole subtree, more the higher they sit
  std::vector<uint32_t> cap(next);
  for (int64_t c = 0; c < next; ++c) {
    if (colleaf[c]) cap[c] = 48u;
    else if (coldepth[c] <= 1) cap[c] = 1024u;
    else if (coldepth[c] == 2) cap[c] = 768u;
    else if (coldepth[c] == 3) cap[c] = 512u;
    else cap[c] = 256u;
  }
  // G entries: a generous multiple of the input, plus the runs a warp may
  // leave partly unused (one per tree node)
  int64_t gcap = std::max<int64_t>(ext.nnz() * 10, 1024) + (int64_t)nodes.size() * GCHUNK;

  cudaDeviceProp prop;
  int dev;
  RCHOL_CUDA(cudaGetDevice(&dev));
  RCHOL_CUDA(cudaGetDeviceProperties(&prop, dev));
  const size_t smem_limit = prop.sharedMemPerBlockOptin;
  RCHOL_CUDA(cudaFuncSetAttribute(eliminate_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem_limit));

  DevBuf<double> diag(next);
  DevBuf<int> flags(NFLAGS);
  for (int attempt = 0; attempt < 12; ++attempt) {
    std::vector<int64_t> base(next + 1, 0);
    for (int64_t c = 0; c < next; ++c) base[c + 1] = base[c] + cap[c];
    DevBuf<uint32_t> fcnt(next), fcap(next);
    DevBuf<int64_t> fbase(next);
    DevBuf<FillRec> frec(std::max<int64_t>(base[next], 1));
    DevBuf<int64_t> gstart(next);
    DevBuf<uint32_t> gcnt(next);
    DevBuf<int32_t> grow(gcap);
    DevBuf<double> gval(gcap);
    DevBuf<unsigned long long> gtop(1);
    RCHOL_CUDA(cudaMemsetAsync(fcnt.p, 0, fcnt.bytes(), s));
    RCHOL_CUDA(cudaMemsetAsync(gcnt.p, 0, gcnt.bytes(), s));
    RCHOL_CUDA(cudaMemsetAsync(gstart.p, 0, gstart.bytes(), s));
    RCHOL_CUDA(cudaMemsetAsync(gtop.p, 0, gtop.bytes(), s));
    RCHOL_CUDA(cudaMemsetAsync(flags.p, 0, flags.bytes(), s));
    fcap.upload(cap.data(), next, s);
    fbase.upload(base.data(), next, s);

    ElimArgs args;
    args.lrp = lrp.p;
    args.lci = lci.p;
    args.lv = lv.p;
    args.lnnz = ext.nnz();
    args.next = next;
    args.fcnt = fcnt.p;
    args.fcap = fcap.p;
    args.fbase = fbase.p;
    args.frec = frec.p;
    args.gstart = gstart.p;
    args.gcnt = gcnt.p;
    args.grow = grow.p;
    args.gval = gval.p;
    args.gtop = gtop.p;
    args.gcap = gcap;
    args.diag = diag.p;
    args.flags = flags.p;
    args.seed = seed;
    std::vector<DevBuf<int64_t>> keep;
    for (int depth = maxdepth; depth >= 1; --depth) {
      std::vector<int64_t> nb, ne;
      int width = 32;
      for (auto &nd : nodes) {
        if (nd.depth != depth || nd.end <= nd.begin) continue;
        nb.push_back(nd.begin);
        ne.push_back(nd.end);
        for (int64_t c = nd.begin; c < nd.end; ++c)
          width = std::max(width, initdeg[c] + (int)cap[c]);
      }
      if (nb.empty()) continue;
      int emax = pow2_at_least(width);
      size_t per_warp = (size_t)emax * 40;
      const bool in_smem = per_warp <= smem_limit;
      int wpb = in_smem ? (int)std::min<size_t>(4, smem_limit / per_warp) : 1;
      keep.emplace_back(nb.size());
      keep.back().upload(nb.data(), nb.size(), s);
      keep.emplace_back(ne.size());
      keep.back().upload(ne.data(), ne.size(), s);
      args.node_begin = keep[keep.size() - 2].p;
      args.node_end = keep.back().p;
      args.num_nodes = (int)nb.size();
      args.emax = emax;
      DevBuf<unsigned char> wide;
      if (!in_smem) wide.alloc(per_warp * nb.size());
      args.gscratch = wide.p;
      int blocks = (int)((nb.size() + wpb - 1) / wpb);
      eliminate_kernel<<<blocks, wpb * 32, in_smem ? per_warp * wpb : 0, s>>>(args);
      RCHOL_CUDA(cudaGetLastError());
      if (!in_smem) RCHOL_CUDA(cudaStreamSynchronize(s));  // `wide` is freed on scope exit
    }
    int hflags[NFLAGS];
    flags.download(hflags, NFLAGS, s);
    RCHOL_CUDA(cudaStreamSynchronize(s));
    if (hflags[FLAG_FILL] || hflags[FLAG_WIDTH]) {
      // Counts past an overflow are lower bounds (truncated columns sample
      // less fill into the columns after them).  Overflowing columns grow to
      // twice their count.  The other columns of an overflowing depth grow
      // to twice the depth's largest count, which settles in one re-run —
      // unless, for the leaves (nearly all columns), that would not fit in
      // 30% of the free device memory (the leaf depth's largest count times
      // 16 million columns took 259 GB at 256^3 on a high-contrast matrix):
      // then every column of an overflowing leaf grows to twice its own
      // count, and further re-runs settle the rest.  Runs repeat until
      // nothing overflows, so the result does not depend on the capacities.
      std::vector<uint32_t> cnt(next);
      fcnt.download(cnt.data(), next, s);
      RCHOL_CUDA(cudaStreamSynchronize(s));
      const int leafd = maxdepth + 1;
      std::vector<uint32_t> depth_max(maxdepth + 2, 0);
      std::vector<char> depth_over(maxdepth + 2, 0), node_over(nodes.size(), 0);
      for (int64_t c = 0; c < next; ++c) {
        const int dd = colleaf[c] ? leafd : coldepth[c];
        depth_max[dd] = std::max(depth_max[dd], cnt[c]);
        if (cnt[c] < cap[c]) continue;
        depth_over[dd] = 1;
        if (colnode[c] >= 0) node_over[colnode[c]] = 1;
      }
      bool leaf_by_depth = true;
      if (depth_over[leafd]) {
        uint64_t recs = 0;
        for (int64_t c = 0; c < next; ++c)
          if (colleaf[c]) recs += std::max<uint64_t>({cap[c], 2ull * cnt[c], 2ull * depth_max[leafd]});
        size_t free_b = 0, total_b = 0;
        RCHOL_CUDA(cudaMemGetInfo(&free_b, &total_b));
        leaf_by_depth = recs * sizeof(FillRec) <= (uint64_t)(0.3 * (double)free_b);
      }
      for (int64_t c = 0; c < next; ++c) {
        const int dd = colleaf[c] ? leafd : coldepth[c];
        if (cnt[c] >= cap[c]) cap[c] = std::max<uint32_t>(cap[c] * 2, cnt[c] * 2);
        if (!depth_over[dd]) continue;
        if (!colleaf[c] || leaf_by_depth) cap[c] = std::max<uint32_t>(cap[c], depth_max[dd] * 2);
        else if (colnode[c] >= 0 && node_over[colnode[c]]) cap[c] = std::max<uint32_t>(cap[c], cnt[c] * 2);
      }
      continue;
    }
    if (hflags[FLAG_GCAP]) {
      gcap *= 2;
      continue;
    }
    if (hflags[FLAG_SINGULAR])
      throw Error(RCHOL_ERR_SINGULAR,
                  "factorization produced a zero pivot (a connected component without "
                  "diagonal excess: the matrix is singular)");
    // ---- assemble U = CSR of G^T --------------------------------------------
    F.n = n;
    F.urp.alloc(n + 1);
    {
      int64_t blocks = (n + 255) / 256;
      u32_to_i64_kernel<<<(unsigned)blocks, 256, 0, s>>>(n, gcnt.p, F.urp.p);
      RCHOL_CUDA(cudaGetLastError());
      exclusive_scan_i64(F.urp.p, n, s);
      int64_t nnz = 0;
      RCHOL_CUDA(cudaMemcpyAsync(&nnz, F.urp.p + n, sizeof(int64_t), cudaMemcpyDeviceToHost, s));
      RCHOL_CUDA(cudaStreamSynchronize(s));
      F.nnz = nnz;
      F.uci.alloc(nnz);
      F.uv.alloc(nnz);
      int64_t threads = n * 32;
      copy_columns_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, s>>>(
          n, gstart.p, gcnt.p, grow.p, gval.p, F.urp.p, F.uci.p, F.uv.p);
      RCHOL_CUDA(cudaGetLastError());
    }
    F.pivots.alloc(n);
    RCHOL_CUDA(cudaMemcpyAsync(F.pivots.p, diag.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    RCHOL_CUDA(cudaStreamSynchronize(s));
    return;
  }
  throw Error(RCHOL_ERR_INTERNAL, "factorization buffers did not converge");
}

}  // namespace rchol
