// rchol oracle: a CPU restatement of the reference's preconditioned-solve
// path, written for checking.  TEST INFRASTRUCTURE ONLY: the product never
// links, loads or calls this file; only tests/, the smoke check and the CPU
// baseline leg of bench.py do.
//
// Parity: pinned.  tests/test_oracle_vs_reference.py checks every routine here
// against the unmodified reference compiled from its own sources
// (oracle/_ref, seeds fixed by oracle/shim/fixed_seed.h), and the committed
// fixtures in tests/golden/ carry those reference outputs to machines that
// have no reference sources.
//
// Two factorization modes share one column routine:
//
//   ORACLE_MODE_REF     reproduces c++/rchol_lap/rchol_lap.cpp bit for bit:
//                       std::mt19937 streams assigned per tree thread exactly
//                       as the reference's std::async tree does, std::sort
//                       tie behaviour, sequential sums.
//   ORACLE_MODE_DEVICE  the contract of the GPU factorization: the same
//                       algorithm with a counter-based Philox4x32-10 stream
//                       keyed by (seed, vertex, sample index), a total order
//                       for every sort, and the summation order of the GPU's
//                       warp scan.  Its output does not depend on the
//                       elimination schedule, so it is computed column by
//                       column in index order.
//
// Build: oracle/Makefile (liboracle.so).  -ffp-contract=off keeps every
// a*b+c rounded twice, as the device code does with explicit _rn intrinsics.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <future>
#include <set>
#include <random>
#include <stdexcept>
#include <string>
#include <thread>
#include <vector>

#include <errno.h>
#include <sys/mman.h>
#include <sys/wait.h>
#include <unistd.h>

#include "shim/metis.h"

namespace {

thread_local std::string g_err;

template <typename T>
T *dup(const T *src, size_t n) {
  T *dst = static_cast<T *>(std::malloc(n ? n * sizeof(T) : sizeof(T)));
  if (n) std::memcpy(dst, src, n * sizeof(T));
  return dst;
}

struct Csr {
  int64_t n = 0;
  std::vector<uint64_t> rp, ci;
  std::vector<double> v;
};

Csr make(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v) {
  Csr a;
  a.n = n;
  a.rp.assign(rp, rp + n + 1);
  a.ci.assign(ci, ci + rp[n]);
  if (v) a.v.assign(v, v + rp[n]);
  return a;
}

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), written from the paper.
// ---------------------------------------------------------------------------
struct U4 {
  uint32_t x[4];
};

U4 philox4x32_10(U4 ctr, uint32_t k0, uint32_t k1) {
  const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
  const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
  for (int r = 0; r < 10; ++r) {
    if (r) {
      k0 += W0;
      k1 += W1;
    }
    uint64_t p0 = (uint64_t)M0 * ctr.x[0];
    uint64_t p1 = (uint64_t)M1 * ctr.x[2];
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    U4 o;
    o.x[0] = hi1 ^ ctr.x[1] ^ k0;
    o.x[1] = lo1;
    o.x[2] = hi0 ^ ctr.x[3] ^ k1;
    o.x[3] = lo0;
    ctr = o;
  }
  return ctr;
}

// Uniform double in [0,1) for sample `i` of vertex `v`: 53 random bits.
double device_uniform(uint64_t seed, uint64_t v, uint64_t i) {
  U4 c;
  c.x[0] = (uint32_t)(i >> 1);
  c.x[1] = 0u;
  c.x[2] = (uint32_t)v;
  c.x[3] = (uint32_t)(v >> 32);
  U4 o = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
  uint32_t a = (i & 1) ? o.x[2] : o.x[0];
  uint32_t b = (i & 1) ? o.x[3] : o.x[1];
  return ((double)(a >> 5) * 67108864.0 + (double)(b >> 6)) * (1.0 / 9007199254740992.0);
}

// ---------------------------------------------------------------------------
// Factorization state: one growable column per vertex of the extended
// Laplacian (c++/rchol_lap/spcol.hpp:6-15 semantics: append-only until the
// column is eliminated).
// ---------------------------------------------------------------------------
struct Column {
  std::vector<uint64_t> row;
  std::vector<double> val;
  std::vector<uint64_t> src;  // device mode: 0 = initial entry, s+1 = fill from s
  size_t split = 0;
};

struct Sample {  // same shape as the reference's sampling record
  uint64_t row;
  double data;
};

struct FillEdge {  // deferred edge: value, row (larger end), col (smaller end)
  double val;
  uint64_t row;
  uint64_t col;
};

struct Factor {
  int64_t next;  // extended size (n + 1)
  std::vector<Column> cols;
  std::vector<double> diag;
  int mode;
  uint64_t seed;
  std::atomic<bool> singular{false};
  size_t par_depth = 0;  // MODE_REF: right children above this depth run on their own thread
};

// c++/rchol_lap/rchol_lap.cpp:794-813: column i from CSR row i of the upper
// extended Laplacian; negative-weight ground entries are skipped.
void load_columns(Factor &F, const Csr &L) {
  F.cols.assign(F.next, Column());
  const uint64_t g = (uint64_t)F.next - 1;
  for (int64_t i = 0; i < F.next; ++i) {
    Column &c = F.cols[i];
    for (uint64_t j = L.rp[i]; j < L.rp[i + 1]; ++j) {
      if (L.ci[j] == g && L.v[j] < 0 && (uint64_t)i != g) continue;
      c.row.push_back(L.ci[j]);
      c.val.push_back(L.v[j]);
      c.src.push_back(0);
    }
    c.split = c.row.size();
  }
}

// c++/rchol_lap/rchol_lap.cpp:733-770 (sort by row, sum duplicates).
void merge_ref(Column &b) {
  size_t size = b.row.size();
  std::vector<Sample> s(size);
  for (size_t i = 0; i < size; ++i) s[i] = Sample{b.row[i], b.val[i]};
  std::sort(s.begin(), s.end(), [](const Sample &x, const Sample &y) { return x.row < y.row; });
  std::vector<uint64_t> r;
  std::vector<double> v;
  r.push_back(s[0].row);
  v.push_back(s[0].data);
  for (size_t i = 1; i < size; ++i) {
    if (s[i].row != r.back()) {
      r.push_back(s[i].row);
      v.push_back(s[i].data);
    } else {
      v.back() += s[i].data;
    }
  }
  b.split = b.row.size() - b.split;
  b.row = r;
  b.val = v;
  b.src.assign(r.size(), 0);
}

// c++/rchol_lap/rchol_lap.cpp:643-729 (random_sampling0), reference order.
double sample_ref(Factor &F, uint64_t c, std::mt19937 &gen, std::vector<FillEdge> &defer,
                  uint64_t lb, uint64_t rb) {
  Column &cur = F.cols[c];
  size_t nz = cur.row.size();
  double sum = 0.0;
  for (size_t i = 1; i < nz; ++i) sum += cur.val[i];
  if (nz > 2) {
    int size = (int)nz - 1;
    std::vector<Sample> s(size);
    std::vector<double> cs(size);
    for (int i = 0; i < size; ++i) s[i] = Sample{cur.row[i + 1], cur.val[i + 1]};
    std::sort(s.begin(), s.end(), [](Sample x, Sample y) { return x.data < y.data; });
    double csum = 0.0;
    for (int i = 0; i < size; ++i) {
      csum += s[i].data;
      cs[i] = csum;
    }
    for (int i = 0; i < size - 1; ++i) {
      std::uniform_real_distribution<> dis(0.0, 1.0);
      double tar = cs[i];
      double r = dis(gen) * (csum - tar) + tar;
      int k = (int)(std::lower_bound(cs.begin() + i, cs.end(), r) - cs.begin());
      if (k >= size) k = size - 1;  // the reference would read past the end
      uint64_t mn = std::min(s[k].row, s[i].row), mx = std::max(s[k].row, s[i].row);
      double w = s[i].data * (csum - cs[i]) / csum;
      if (mn >= lb && mn < rb) {
        F.cols[mn].row.push_back(mx);
        F.cols[mn].val.push_back(w);
        F.cols[mn].src.push_back(0);
      } else {
        defer.push_back(FillEdge{w, mx, mn});
      }
    }
  }
  double inv = 1.0 / sum;
  for (size_t i = 0; i < nz; ++i) cur.val[i] *= inv;
  cur.val[0] = 1.0;
  if (!(sum > 0.0) && (int64_t)c != F.next - 1) F.singular = true;
  return sum;
}

void eliminate_ref(Factor &F, uint64_t c, std::mt19937 &gen, std::vector<FillEdge> &defer,
                   uint64_t lb, uint64_t rb) {
  Column &b = F.cols[c];
  if (b.row.size() - b.split > 0) merge_ref(b);
  F.diag[c] = sample_ref(F, c, gen, defer, lb, rb);
}

// c++/rchol_lap/rchol_lap.cpp:187-355.  `gen` is the sampler of the OS thread
// that runs this node in the reference: the right child gets a fresh thread
// (std::async, :254) and therefore a freshly seeded generator; the left child
// and the separator run on the current thread.
std::vector<FillEdge> tree_ref(Factor &F, const std::vector<uint64_t> &ri, size_t depth,
                               size_t start, size_t total, size_t target, std::mt19937 &gen) {
  std::vector<FillEdge> defer;
  if (depth == target) {
    uint64_t lb = ri[start], rb = ri[start + total];
    for (uint64_t i = lb; i < rb; ++i) eliminate_ref(F, i, gen, defer, lb, rb);
    return defer;
  }
  // The two subtrees touch disjoint columns, so the right one may run on a
  // thread of its own, as the reference's std::async does (near the root
  // only, to bound the thread count); the streams and results are the same
  // either way.
  auto right = [&F, &ri, depth, start, total, target] {
    std::mt19937 rgen((std::mt19937::result_type)F.seed);
    return tree_ref(F, ri, depth + 1, (total - 1) / 2 + start, (total - 1) / 2, target, rgen);
  };
  std::vector<FillEdge> r, l;
  if (depth <= F.par_depth) {
    std::future<std::vector<FillEdge>> fr = std::async(std::launch::async, right);
    l = tree_ref(F, ri, depth + 1, start, (total - 1) / 2, target, gen);
    r = fr.get();
  } else {
    r = right();
    l = tree_ref(F, ri, depth + 1, start, (total - 1) / 2, target, gen);
  }
  uint64_t lb = ri[start + total - 1], rb = ri[start + total];
  for (const std::vector<FillEdge> *part : {&l, &r}) {
    for (const FillEdge &e : *part) {
      if (e.col >= lb && e.col < rb) {
        F.cols[e.col].row.push_back(e.row);
        F.cols[e.col].val.push_back(e.val);
        F.cols[e.col].src.push_back(0);
      } else {
        defer.push_back(e);
      }
    }
  }
  for (uint64_t i = lb; i < rb; ++i) eliminate_ref(F, i, gen, defer, lb, rb);
  return defer;
}

// ---------------------------------------------------------------------------
// Device-contract column elimination.
// ---------------------------------------------------------------------------

// Inclusive prefix sum in the order of a 32-lane Hillis-Steele warp scan
// (offsets 1,2,4,8,16), chunk by chunk, each chunk offset by the running
// total of the previous ones.
void warp_order_scan(const std::vector<double> &w, std::vector<double> &cs) {
  size_t m = w.size();
  cs.assign(m, 0.0);
  double carry = 0.0;
  for (size_t base = 0; base < m; base += 32) {
    double v[32];
    for (int l = 0; l < 32; ++l) v[l] = (base + l < m) ? w[base + l] : 0.0;
    for (int d = 1; d < 32; d <<= 1) {
      double nv[32];
      for (int l = 0; l < 32; ++l) nv[l] = (l >= d) ? v[l - d] + v[l] : v[l];
      std::memcpy(v, nv, sizeof(v));
    }
    for (int l = 0; l < 32 && base + l < m; ++l) cs[base + l] = carry + v[l];
    carry = cs[std::min(m, base + 32) - 1];
  }
}

// Column statistics of the last device-mode factorization (entries before the
// merge, incoming fill, merged length), for sizing the device buffers.
std::vector<uint32_t> g_stat_entries, g_stat_fill, g_stat_merged;

void eliminate_device(Factor &F, uint64_t c) {
  Column &col = F.cols[c];
  if (g_stat_entries.size() != (size_t)F.next) {
    g_stat_entries.assign(F.next, 0);
    g_stat_fill.assign(F.next, 0);
    g_stat_merged.assign(F.next, 0);
  }
  g_stat_entries[c] = (uint32_t)col.row.size();
  g_stat_fill[c] = (uint32_t)(col.row.size() - col.split);
  // 1. merge: order by (row, source), sum duplicate rows left to right, drop
  //    the diagonal (row == c), which the reference overwrites anyway.
  size_t nz = col.row.size();
  std::vector<size_t> ord(nz);
  for (size_t i = 0; i < nz; ++i) ord[i] = i;
  std::sort(ord.begin(), ord.end(), [&](size_t a, size_t b) {
    if (col.row[a] != col.row[b]) return col.row[a] < col.row[b];
    return col.src[a] < col.src[b];
  });
  std::vector<uint64_t> rows;
  std::vector<double> w;
  for (size_t t = 0; t < nz; ++t) {
    size_t i = ord[t];
    if (col.row[i] == c) continue;
    if (!rows.empty() && rows.back() == col.row[i]) {
      w.back() = w.back() + col.val[i];
    } else {
      rows.push_back(col.row[i]);
      w.push_back(col.val[i]);
    }
  }
  size_t m = rows.size();
  g_stat_merged[c] = (uint32_t)m;
  // 2. order by (weight, row) and scan.
  std::vector<size_t> o2(m);
  for (size_t i = 0; i < m; ++i) o2[i] = i;
  std::sort(o2.begin(), o2.end(), [&](size_t a, size_t b) {
    if (w[a] != w[b]) return w[a] < w[b];
    return rows[a] < rows[b];
  });
  std::vector<double> ws(m), cs;
  std::vector<uint64_t> rs(m);
  for (size_t i = 0; i < m; ++i) {
    ws[i] = w[o2[i]];
    rs[i] = rows[o2[i]];
  }
  warp_order_scan(ws, cs);
  double csum = m ? cs[m - 1] : 0.0;
  // 3. sample m-1 fill edges; self loops are dropped (they would only merge
  //    into the target's diagonal).
  for (size_t i = 0; i + 1 < m; ++i) {
    double u = device_uniform(F.seed, c, i);
    double tar = cs[i];
    double span = csum - tar;
    double r = u * span;
    r = r + tar;
    size_t k = (size_t)(std::lower_bound(cs.begin() + i, cs.end(), r) - cs.begin());
    if (k >= m) k = m - 1;
    if (k == i) continue;
    double wn = ws[i] * span;
    wn = wn / csum;
    uint64_t mn = std::min(rs[i], rs[k]), mx = std::max(rs[i], rs[k]);
    Column &t = F.cols[mn];
    t.row.push_back(mx);
    t.val.push_back(wn);
    t.src.push_back(c + 1);
  }
  // 4. the column of G (before the sqrt(d) scaling): rows ascending.
  col.row.assign(1, c);
  col.val.assign(1, 1.0);
  col.src.assign(1, 0);
  double inv = 1.0 / csum;
  for (size_t i = 0; i < m; ++i) {
    col.row.push_back(rows[i]);
    col.val.push_back(w[i] * inv);
    col.src.push_back(0);
  }
  F.diag[c] = csum;
  if (!(csum > 0.0) && (int64_t)c != F.next - 1) F.singular = true;
}

// c++/rchol_lap/rchol_lap.cpp:358-387 (coalesce): CSR of G^T, ground row
// dropped, off-diagonals negated, every column scaled by sqrt(d).
void coalesce(const Factor &F, std::vector<uint64_t> &rp, std::vector<uint64_t> &ci,
              std::vector<double> &v) {
  int64_t m = F.next - 1;
  rp.assign(m + 1, 0);
  ci.clear();
  v.clear();
  for (int64_t i = 0; i < m; ++i) {
    const Column &c = F.cols[i];
    double sq = std::sqrt(F.diag[i]);
    for (size_t j = 0; j < c.row.size(); ++j) {
      if (c.row[j] == (uint64_t)m) continue;
      double x = c.val[j];
      if (c.row[j] != (uint64_t)i) x = x * -1;
      x *= sq;
      ci.push_back(c.row[j]);
      v.push_back(x);
    }
    rp[i + 1] = ci.size();
  }
}

// ---------------------------------------------------------------------------
// Ordering: c++/rchol/find_separator.cpp:5-163 restated.
// ---------------------------------------------------------------------------
std::vector<int64_t> metis_sep(const Csr &A) {
  idx_t N = A.n;
  std::vector<idx_t> xadj(A.rp.begin(), A.rp.end()), adj(A.ci.begin(), A.ci.end());
  std::vector<idx_t> part(N > 0 ? N : 1, 0);
  idx_t sepsize = 1;
  METIS_ComputeVertexSeparator(&N, xadj.data(), adj.data(), nullptr, nullptr, &sepsize,
                               part.data());
  return std::vector<int64_t>(part.begin(), part.begin() + N);
}

Csr submatrix(const std::vector<uint64_t> &par, const std::vector<int64_t> &sep, const Csr &A) {
  std::vector<uint64_t> tr(A.n, 0);
  for (size_t i = 0; i < par.size(); ++i) tr[par[i]] = i;
  Csr B;
  B.n = (int64_t)par.size();
  B.rp.push_back(0);
  int64_t lab = par.empty() ? -1 : sep[par[0]];
  for (uint64_t u : par) {
    uint64_t cnt = 0;
    for (uint64_t j = A.rp[u]; j < A.rp[u + 1]; ++j) {
      if (sep[A.ci[j]] == lab) {
        B.ci.push_back(tr[A.ci[j]]);
        ++cnt;
      }
    }
    B.rp.push_back(B.rp.back() + cnt);
  }
  return B;
}

// last_in_root: python/rchol_lap/find_separator.pyx:27-28 (the Python front
// end forces the last vertex into the root separator).
// Leaf order (no counterpart in the C++ reference, which keeps the natural
// order; the MATLAB front end uses amd, matlab/rchol/find_separator.m:6):
// 1 = METIS_NodeND, 2 = minimum degree (least degree in the elimination
// graph first, ties by lowest index, neighbours joined into a clique).
std::vector<uint64_t> leaf_order_of(const Csr &A, int mode) {
  const int64_t n = A.n;
  std::vector<uint64_t> p(n);
  for (int64_t i = 0; i < n; ++i) p[i] = (uint64_t)i;
  if (mode == 0 || n <= 2) return p;
  if (mode == 1) {
    idx_t N = n;
    std::vector<idx_t> xadj(A.rp.begin(), A.rp.end()), adj(A.ci.begin(), A.ci.end()), perm(n), iperm(n);
    if (adj.empty()) adj.push_back(0);
    METIS_NodeND(&N, xadj.data(), adj.data(), nullptr, nullptr, perm.data(), iperm.data());
    for (int64_t i = 0; i < n; ++i) p[i] = (uint64_t)perm[i];
    return p;
  }
  std::vector<std::set<int64_t>> nb(n);
  for (int64_t i = 0; i < n; ++i)
    for (uint64_t j = A.rp[i]; j < A.rp[i + 1]; ++j)
      if ((int64_t)A.ci[j] != i) nb[i].insert((int64_t)A.ci[j]);
  std::vector<char> gone(n, 0);
  for (int64_t k = 0; k < n; ++k) {
    int64_t v = -1;
    for (int64_t i = 0; i < n; ++i)  // least degree, lowest index
      if (!gone[i] && (v < 0 || nb[i].size() < nb[v].size())) v = i;
    p[k] = (uint64_t)v;
    gone[v] = 1;
    std::vector<int64_t> N(nb[v].begin(), nb[v].end());
    for (int64_t u : N) {
      nb[u].erase(v);
      for (int64_t w : N)
        if (w != u) nb[u].insert(w);
    }
    nb[v].clear();
  }
  return p;
}

void find_sep(const Csr &A, int depth, int target, std::vector<uint64_t> &p,
              std::vector<uint64_t> &val, bool last_in_root = false, int leaf = 0, int forks = 0);

// Orders subgraph R in a forked child process while the caller orders the
// other half.  The METIS archive keeps its state in process globals, so
// threads would perturb each other; a child has its own copy, and every
// METIS call still sees exactly the subgraph of the serial recursion, so the
// ordering is unchanged.  Returns false (nothing started) if fork fails.
struct ForkedSep {
  pid_t pid = -1;
  uint64_t *shm = nullptr;
  size_t bytes = 0;
};

bool fork_sep(const Csr &R, int depth, int target, int leaf, int forks, ForkedSep &f) {
  const size_t nseg = ((size_t)1 << (target - depth + 1)) - 1;  // segments below `depth`
  f.bytes = (2 + (size_t)R.n + nseg) * sizeof(uint64_t);
  void *m = mmap(nullptr, f.bytes, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
  if (m == MAP_FAILED) return false;
  f.shm = static_cast<uint64_t *>(m);
  f.shm[0] = 2;  // status: 0 ok, 1 invalid argument, 2 failure
  f.pid = fork();
  if (f.pid < 0) {
    munmap(m, f.bytes);
    return false;
  }
  if (f.pid == 0) {
    uint64_t st = 2;
    try {
      std::vector<uint64_t> pr, vr;
      find_sep(R, depth, target, pr, vr, false, leaf, forks);
      if (vr.size() <= nseg) {
        std::memcpy(f.shm + 2, pr.data(), pr.size() * sizeof(uint64_t));
        std::memcpy(f.shm + 2 + R.n, vr.data(), vr.size() * sizeof(uint64_t));
        f.shm[1] = vr.size();
        st = 0;
      }
    } catch (const std::invalid_argument &) {
      st = 1;
    } catch (...) {
    }
    f.shm[0] = st;
    _exit(0);
  }
  return true;
}

void join_sep(ForkedSep &f, int64_t n, std::vector<uint64_t> &pr, std::vector<uint64_t> &vr) {
  int st = 0;
  while (waitpid(f.pid, &st, 0) < 0 && errno == EINTR) {
  }
  const uint64_t status = f.shm[0];
  if (status == 0) {
    pr.assign(f.shm + 2, f.shm + 2 + n);
    vr.assign(f.shm + 2 + n, f.shm + 2 + n + f.shm[1]);
  }
  munmap(f.shm, f.bytes);
  if (status == 1) throw std::invalid_argument("too many threads requested");
  if (status != 0) throw std::runtime_error("ordering worker process failed");
}

void find_sep(const Csr &A, int depth, int target, std::vector<uint64_t> &p,
              std::vector<uint64_t> &val, bool last_in_root, int leaf, int forks) {
  if (depth == target) {
    val.assign(1, (uint64_t)A.n);
    p = leaf_order_of(A, leaf);
    return;
  }
  if (A.n <= 1) throw std::invalid_argument("too many threads requested");
  std::vector<int64_t> sep = metis_sep(A);
  if (last_in_root && depth == 1) sep[A.n - 1] = 2;
  std::vector<uint64_t> l, r, s;
  for (int64_t i = 0; i < A.n; ++i) {
    if (sep[i] == 0) l.push_back(i);
    else if (sep[i] == 1) r.push_back(i);
    else s.push_back(i);
  }
  Csr L = submatrix(l, sep, A), R = submatrix(r, sep, A);
  std::vector<uint64_t> pl, vl, pr, vr;
  ForkedSep f;
  if (forks > 0 && R.n >= 20000 && fork_sep(R, depth + 1, target, leaf, forks - 1, f)) {
    try {
      find_sep(L, depth + 1, target, pl, vl, false, leaf, forks - 1);
    } catch (...) {
      try {
        join_sep(f, R.n, pr, vr);
      } catch (...) {
      }
      throw;
    }
    join_sep(f, R.n, pr, vr);
  } else {
    find_sep(L, depth + 1, target, pl, vl, false, leaf, forks);
    find_sep(R, depth + 1, target, pr, vr, false, leaf, forks);
  }
  val = vl;
  val.insert(val.end(), vr.begin(), vr.end());
  val.push_back(s.size());
  p.clear();
  for (uint64_t x : pl) p.push_back(l[x]);
  for (uint64_t x : pr) p.push_back(r[x]);
  p.insert(p.end(), s.begin(), s.end());
}

// c++/util/util.cpp:16-49
Csr reorder(const Csr &A, const std::vector<uint64_t> &perm) {
  int64_t n = (int64_t)perm.size();
  std::vector<uint64_t> tr(n);
  for (int64_t i = 0; i < n; ++i) tr[perm[i]] = i;
  Csr B;
  B.n = n;
  B.rp.push_back(0);
  for (int64_t i = 0; i < n; ++i) {
    uint64_t a = A.rp[perm[i]], b = A.rp[perm[i] + 1];
    std::vector<Sample> s;
    for (uint64_t j = a; j < b; ++j) s.push_back(Sample{tr[A.ci[j]], A.v[j]});
    std::sort(s.begin(), s.end(), [](const Sample &x, const Sample &y) { return x.row < y.row; });
    for (const Sample &e : s) {
      B.ci.push_back(e.row);
      B.v.push_back(e.data);
    }
    B.rp.push_back(B.ci.size());
  }
  return B;
}

// c++/util/util.hpp:60-142 then :85-91 (triu, ground vertex, negate).
Csr extend(const Csr &A) {
  int64_t n = A.n;
  Csr L;
  L.n = n + 1;
  L.rp.assign(n + 2, 0);
  double overall = 0.0;
  for (int64_t r = 0; r < n; ++r) {
    for (uint64_t j = A.rp[r]; j < A.rp[r + 1]; ++j) {
      if ((uint64_t)r <= A.ci[j]) {
        L.ci.push_back(A.ci[j]);
        L.v.push_back(A.v[j]);
      }
    }
    double sum = 0.0;
    for (uint64_t j = A.rp[r]; j < A.rp[r + 1]; ++j) sum += A.v[j];
    if (std::abs(sum) > 1e-09) {
      L.ci.push_back((uint64_t)n);
      L.v.push_back(-sum);
    }
    L.rp[r + 1] = L.ci.size();
    overall -= sum;
  }
  if (std::abs(overall) > 1e-09) {
    L.ci.push_back((uint64_t)n);
    L.v.push_back(-overall);
  }
  L.rp[n + 1] = L.ci.size();
  for (double &x : L.v) x *= -1;
  return L;
}

void export_csr(const std::vector<uint64_t> &rp, const std::vector<uint64_t> &ci,
                const std::vector<double> &v, uint64_t **orp, uint64_t **oci, double **ov) {
  *orp = dup(rp.data(), rp.size());
  *oci = dup(ci.data(), ci.size());
  *ov = dup(v.data(), v.size());
}

// c++/util/pcg.cpp:141-159 with the serial triangular solves of the MKL
// stand-in: forward sweep with U^T (U = CSR of G^T), then backward with U.
void precond(const Csr &U, const double *r, double *z, std::vector<double> &y) {
  int64_t n = U.n;
  y.assign(r, r + n);
  for (int64_t i = 0; i < n; ++i) {
    double d = 0.0;
    for (uint64_t k = U.rp[i]; k < U.rp[i + 1]; ++k)
      if (U.ci[k] == (uint64_t)i) d = U.v[k];
    y[i] /= d;
    for (uint64_t k = U.rp[i]; k < U.rp[i + 1]; ++k)
      if (U.ci[k] > (uint64_t)i) y[U.ci[k]] -= U.v[k] * y[i];
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    double acc = y[i], d = 0.0;
    for (uint64_t k = U.rp[i]; k < U.rp[i + 1]; ++k) {
      if (U.ci[k] == (uint64_t)i) d = U.v[k];
      else if (U.ci[k] > (uint64_t)i) acc -= U.v[k] * z[U.ci[k]];
    }
    z[i] = acc / d;
  }
}

// The same two solves in another valid FP64 evaluation order: the forward
// sweep in dot form over the rows of G (each row's terms summed from its last
// column down), the backward sweep summing each row from its last column.
// Used only to measure how far the reference PCG itself moves when nothing
// but the rounding order changes.
void precond_alt(const Csr &U, const Csr &L, const double *r, double *z, std::vector<double> &y) {
  int64_t n = U.n;
  y.assign(n, 0.0);
  for (int64_t i = 0; i < n; ++i) {
    double acc = 0.0, d = 0.0;
    for (uint64_t k = L.rp[i + 1]; k-- > L.rp[i];) {
      if (L.ci[k] == (uint64_t)i) d = L.v[k];
      else if (L.ci[k] < (uint64_t)i) acc += L.v[k] * y[L.ci[k]];
    }
    y[i] = (r[i] - acc) / d;
  }
  for (int64_t i = n - 1; i >= 0; --i) {
    double acc = 0.0, d = 0.0;
    for (uint64_t k = U.rp[i + 1]; k-- > U.rp[i];) {
      if (U.ci[k] == (uint64_t)i) d = U.v[k];
      else if (U.ci[k] > (uint64_t)i) acc += U.v[k] * z[U.ci[k]];
    }
    z[i] = (y[i] - acc) / d;
  }
}

Csr transpose(const Csr &U) {
  Csr L;
  L.n = U.n;
  L.rp.assign(U.n + 1, 0);
  for (uint64_t k = 0; k < U.rp[U.n]; ++k) ++L.rp[U.ci[k] + 1];
  for (int64_t i = 0; i < U.n; ++i) L.rp[i + 1] += L.rp[i];
  L.ci.resize(U.rp[U.n]);
  L.v.resize(U.rp[U.n]);
  std::vector<uint64_t> cur(L.rp.begin(), L.rp.end() - 1);
  for (int64_t i = 0; i < U.n; ++i)
    for (uint64_t k = U.rp[i]; k < U.rp[i + 1]; ++k) {
      const uint64_t w = cur[U.ci[k]]++;
      L.ci[w] = (uint64_t)i;
      L.v[w] = U.v[k];
    }
  return L;
}

void spmv(const Csr &A, const double *x, double *y, int threads) {
#pragma omp parallel for schedule(static) num_threads(threads) if (threads > 1)
  for (int64_t i = 0; i < A.n; ++i) {
    double s = 0.0;
    for (uint64_t k = A.rp[i]; k < A.rp[i + 1]; ++k) s += A.v[k] * x[A.ci[k]];
    y[i] = s;
  }
}

double dot(int64_t n, const double *x, const double *y, int threads) {
  double s = 0.0;
  if (threads > 1) {
#pragma omp parallel for reduction(+ : s) schedule(static) num_threads(threads)
    for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
  } else {
    for (int64_t i = 0; i < n; ++i) s += x[i] * y[i];
  }
  return s;
}

}  // namespace

extern "C" {

const char *oracle_last_error() { return g_err.c_str(); }
void oracle_free(void *p) { std::free(p); }

// c++/util/laplace_3d.hpp:8-61: 7-point Dirichlet Laplacian, k fastest.
int oracle_laplace_3d(int64_t n, uint64_t **rp, uint64_t **ci, double **v) {
  std::vector<uint64_t> r{0}, c;
  std::vector<double> x;
  int64_t n2 = n * n;
  for (int64_t i = 0; i < n; ++i)
    for (int64_t j = 0; j < n; ++j)
      for (int64_t k = 0; k < n; ++k) {
        int64_t id = k + j * n + i * n2;
        auto put = [&](int64_t col, double val) {
          c.push_back((uint64_t)col);
          x.push_back(val);
        };
        if (i > 0) put(id - n2, -1);
        if (j > 0) put(id - n, -1);
        if (k > 0) put(id - 1, -1);
        put(id, 6);
        if (k < n - 1) put(id + 1, -1);
        if (j < n - 1) put(id + n, -1);
        if (i < n - 1) put(id + n2, -1);
        r.push_back(c.size());
      }
  export_csr(r, c, x, rp, ci, v);
  return 0;
}

int oracle_extend(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v,
                  uint64_t **orp, uint64_t **oci, double **ov) {
  Csr L = extend(make(n, rp, ci, v));
  export_csr(L.rp, L.ci, L.v, orp, oci, ov);
  return 0;
}

int oracle_reorder(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v,
                   const uint64_t *perm, uint64_t **orp, uint64_t **oci, double **ov) {
  Csr B = reorder(make(n, rp, ci, v), std::vector<uint64_t>(perm, perm + n));
  export_csr(B.rp, B.ci, B.v, orp, oci, ov);
  return 0;
}

// c++/rchol/rchol_parallel.cpp:37-70: remove the diagonal, nested dissection
// to depth log2(threads)+1, result_idx with the ground vertex in the root.
// flags: 1 = last vertex in the root separator (Python front end), 2 = leaf
// order METIS_NodeND, 4 = leaf order minimum degree.
int oracle_order_ex(int64_t n, const uint64_t *rp, const uint64_t *ci, int threads, int flags,
                    uint64_t **perm, uint64_t **ridx, int64_t *nridx) {
  try {
    if (threads <= 0) throw std::invalid_argument("thread number should be positive");
    if ((threads & (threads - 1)) != 0)
      throw std::invalid_argument("thread number should be a power of 2");
    Csr A;
    A.n = n;
    A.rp.push_back(0);
    for (int64_t i = 0; i < n; ++i) {
      for (uint64_t j = rp[i]; j < rp[i + 1]; ++j)
        if (ci[j] != (uint64_t)i) A.ci.push_back(ci[j]);
      A.rp.push_back(A.ci.size());
    }
    int target = 1;
    while ((1 << (target - 1)) < threads) ++target;
    std::vector<uint64_t> p, val;
    int forks = 0;  // levels of the recursion that order their right half in a child process
    while ((1u << forks) < std::max(1u, std::thread::hardware_concurrency())) ++forks;
    if (const char *e = std::getenv("ORACLE_ORDER_FORK_LEVELS")) forks = std::atoi(e);
    find_sep(A, 1, target, p, val, (flags & 1) != 0, (flags & 2) ? 1 : (flags & 4) ? 2 : 0, forks);
    std::vector<uint64_t> ri{0};
    for (uint64_t x : val) ri.push_back(ri.back() + x);
    ri.back() += 1;
    *perm = dup(p.data(), p.size());
    *ridx = dup(ri.data(), ri.size());
    *nridx = (int64_t)ri.size();
    return 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

int oracle_order(int64_t n, const uint64_t *rp, const uint64_t *ci, int threads,
                 uint64_t **perm, uint64_t **ridx, int64_t *nridx) {
  return oracle_order_ex(n, rp, ci, threads, 0, perm, ridx, nridx);
}

// Factor the extended Laplacian L (upper CSR, positive edge weights, as
// produced by oracle_extend).  ridx is the tree partition (result_idx).
// Outputs G as CSR of G^T and, if d is non-null, the pivots d (length next).
int oracle_factor(int64_t next, const uint64_t *rp, const uint64_t *ci, const double *v,
                  const uint64_t *ridx, int64_t nridx, int mode, uint64_t seed,
                  uint64_t **grp, uint64_t **gci, double **gv, double *d) {
  try {
    Csr L = make(next, rp, ci, v);
    Factor F;
    F.next = next;
    F.mode = mode;
    F.seed = seed;
    F.diag.assign(next, 0.0);
    load_columns(F, L);
    if (mode == 0) {
      std::vector<uint64_t> ri(ridx, ridx + nridx);
      size_t threads = ri.size() / 2;
      size_t target = (size_t)(std::log2((double)threads) + 1);
      const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
      F.par_depth = (size_t)std::log2((double)hw);  // about one thread per core
      std::mt19937 gen((std::mt19937::result_type)seed);
      tree_ref(F, ri, 1, 0, ri.size() - 1, target, gen);
    } else {
      for (int64_t c = 0; c < next; ++c) eliminate_device(F, (uint64_t)c);
    }
    std::vector<uint64_t> orp, oci;
    std::vector<double> ov;
    coalesce(F, orp, oci, ov);
    export_csr(orp, oci, ov, grp, gci, gv);
    if (d) std::memcpy(d, F.diag.data(), next * sizeof(double));
    return F.singular ? 2 : 0;
  } catch (const std::exception &e) {
    g_err = e.what();
    return 1;
  }
}

// z = (G G^T)^{-1} r with G given as CSR of G^T.
int oracle_precond(int64_t n, const uint64_t *grp, const uint64_t *gci, const double *gv,
                   const double *r, double *z) {
  Csr U = make(n, grp, gci, gv);
  std::vector<double> y;
  precond(U, r, z, y);
  return 0;
}

// Forward solve only: y = G^{-1} r.
int oracle_trsv_lower(int64_t n, const uint64_t *grp, const uint64_t *gci, const double *gv,
                      const double *r, double *y) {
  Csr U = make(n, grp, gci, gv);
  std::vector<double> t(r, r + n);
  for (int64_t i = 0; i < n; ++i) {
    double d = U.v[U.rp[i]];
    for (uint64_t k = U.rp[i]; k < U.rp[i + 1]; ++k)
      if (U.ci[k] == (uint64_t)i) d = U.v[k];
    t[i] /= d;
    for (uint64_t k = U.rp[i]; k < U.rp[i + 1]; ++k)
      if (U.ci[k] > (uint64_t)i) t[U.ci[k]] -= U.v[k] * t[i];
  }
  std::memcpy(y, t.data(), n * sizeof(double));
  return 0;
}

// Backward solve only: z = G^{-T} y.
int oracle_trsv_upper(int64_t n, const uint64_t *grp, const uint64_t *gci, const double *gv,
                      const double *y, double *z) {
  Csr U = make(n, grp, gci, gv);
  for (int64_t i = n - 1; i >= 0; --i) {
    double acc = y[i], d = 0.0;
    for (uint64_t k = U.rp[i]; k < U.rp[i + 1]; ++k) {
      if (U.ci[k] == (uint64_t)i) d = U.v[k];
      else if (U.ci[k] > (uint64_t)i) acc -= U.v[k] * z[U.ci[k]];
    }
    z[i] = acc / d;
  }
  return 0;
}

int oracle_spmv(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v,
                const double *x, double *y) {
  Csr A = make(n, rp, ci, v);
  spmv(A, x, y, 1);
  return 0;
}

// c++/util/pcg.cpp:57-127.  With threads == 1 the arithmetic follows the
// serial MKL stand-in exactly; threads > 1 parallelises SpMV (same per-row
// order) and the dot products (different summation order); threads < 0 uses
// |threads| threads and also the other evaluation order of the triangular
// solves (precond_alt).  The last two only measure rounding sensitivity.  If
// hist is non-null, ||r_k|| / ||b|| after each iteration k is stored in
// hist[k].
int oracle_pcg(int64_t n, const uint64_t *rp, const uint64_t *ci, const double *v,
               const double *b, double tol, int maxit, const uint64_t *grp,
               const uint64_t *gci, const double *gv, int threads, double *x,
               double *relres, int *itr, double *hist) {
  Csr A = make(n, rp, ci, v);
  Csr U = make(n, grp, gci, gv);
  const bool alt = threads < 0;
  threads = std::abs(threads);
  Csr L;
  if (alt) L = transpose(U);
  std::vector<double> r(b, b + n), pr(n, 0.0), pz(n, 0.0), p(n, 0.0), z(n, 0.0), q(n, 0.0), y;
  std::fill(x, x + n, 0.0);
  double nb = std::sqrt(dot(n, b, b, threads));
  int it = 0;
  while (std::sqrt(dot(n, r.data(), r.data(), threads)) > nb * tol && it < maxit) {
    if (alt) precond_alt(U, L, r.data(), z.data(), y);
    else precond(U, r.data(), z.data(), y);
    if (it == 0) {
      p = z;
    } else {
      double d1 = dot(n, r.data(), z.data(), threads);
      double d2 = dot(n, pr.data(), pz.data(), threads);
      double beta = d1 / d2;
      for (int64_t i = 0; i < n; ++i) p[i] *= beta;
      for (int64_t i = 0; i < n; ++i) p[i] += 1 * z[i];
    }
    spmv(A, p.data(), q.data(), threads);
    double d1 = dot(n, p.data(), r.data(), threads);
    double d2 = dot(n, p.data(), q.data(), threads);
    double alpha = d1 / d2;
    for (int64_t i = 0; i < n; ++i) x[i] += alpha * p[i];
    pr = r;
    pz = z;
    for (int64_t i = 0; i < n; ++i) r[i] += -alpha * q[i];
    ++it;
    if (hist) hist[it - 1] = std::sqrt(dot(n, r.data(), r.data(), threads)) / nb;
  }
  spmv(A, x, q.data(), threads);
  for (int64_t i = 0; i < n; ++i) q[i] += -1 * b[i];
  *relres = std::sqrt(dot(n, q.data(), q.data(), threads)) / nb;
  *itr = it;
  return 0;
}

// Philox known-answer hook: writes the 4 output words for (ctr, key).
void oracle_philox(const uint32_t *ctr, const uint32_t *key, uint32_t *out) {
  U4 c;
  for (int i = 0; i < 4; ++i) c.x[i] = ctr[i];
  U4 o = philox4x32_10(c, key[0], key[1]);
  for (int i = 0; i < 4; ++i) out[i] = o.x[i];
}

double oracle_uniform(uint64_t seed, uint64_t v, uint64_t i) { return device_uniform(seed, v, i); }

// Per-column statistics of the last device-mode factorization on this thread:
// entries before the merge, incoming fill entries, merged off-diagonal count.
int64_t oracle_column_stats(uint32_t *entries, uint32_t *fill, uint32_t *merged, int64_t cap) {
  int64_t n = (int64_t)g_stat_entries.size();
  if (entries && cap >= n) {
    std::memcpy(entries, g_stat_entries.data(), n * 4);
    std::memcpy(fill, g_stat_fill.data(), n * 4);
    std::memcpy(merged, g_stat_merged.data(), n * 4);
  }
  return n;
}

}  // extern "C"
