// Host side of the solve path: nested-dissection ordering with METIS, the
// permuted matrix A(p,p), the extended Laplacian handed to the GPU
// factorization, and the separator tree.  Everything here is integer or
// layout work that must agree bit for bit with the reference.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <exception>
#include <functional>
#include <memory>
#include <mutex>
#include <future>
#include <numeric>
#include <set>
#include <thread>

#include <errno.h>
#include <sys/mman.h>
#include <sys/wait.h>
#include <unistd.h>

#include "common.hpp"
#include "host.hpp"

// METIS 5 as shipped in the CUDA toolkit (libmetis_static.a, 64-bit idx_t).
extern "C" int METIS_ComputeVertexSeparator(int64_t *nvtxs, int64_t *xadj, int64_t *adjncy,
                                            int64_t *vwgt, int64_t *options, int64_t *sepsize,
                                            int64_t *part);
extern "C" int METIS_NodeND(int64_t *nvtxs, int64_t *xadj, int64_t *adjncy, int64_t *vwgt, int64_t *options,
                            int64_t *perm, int64_t *iperm);

namespace rchol {

int host_threads() {
  unsigned h = std::thread::hardware_concurrency();
  return h ? (int)std::min(h, 64u) : 4;
}

// Blocks of at least `grain` indices (and about 16 per thread) handed out in
// order to the threads as they come free, so that uneven work (large and
// small pieces of a solve plan) spreads over all threads.  The first
// exception thrown by any block is rethrown to the caller after all threads
// have stopped taking blocks.
void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)> &body, int64_t grain) {
  const int T = host_threads();
  if (n <= grain || T <= 1) {
    body(0, n);
    return;
  }
  const int64_t block = std::max<int64_t>(std::max<int64_t>(grain, 1), (n + 16 * (int64_t)T - 1) / (16 * (int64_t)T));
  const int64_t nblocks = (n + block - 1) / block;
  std::atomic<int64_t> next{0};
  std::atomic<bool> failed{false};
  std::exception_ptr first;
  std::mutex mu;
  auto worker = [&]() {
    for (;;) {
      const int64_t b = next.fetch_add(1);
      if (b >= nblocks || failed.load()) return;
      try {
        body(b * block, std::min(n, (b + 1) * block));
      } catch (...) {
        std::lock_guard<std::mutex> lk(mu);
        if (!first) first = std::current_exception();
        failed.store(true);
        return;
      }
    }
  };
  std::vector<std::thread> th;
  const int64_t nt = std::min<int64_t>(T, nblocks);
  for (int64_t t = 1; t < nt; ++t) th.emplace_back(worker);
  worker();
  for (auto &t : th) t.join();
  if (first) std::rethrow_exception(first);
}

namespace {

// Adjacency structure without the diagonal (c++/rchol/rchol_parallel.cpp:9-34),
// in METIS's own index type.
struct Graph {
  int64_t n = 0;
  std::vector<int64_t> xadj, adj;
};

std::vector<int64_t> metis_separator(Graph &g) {
  int64_t N = g.n, sepsize = 1;
  std::vector<int64_t> part(N > 0 ? N : 1, 0);
  int rc = METIS_ComputeVertexSeparator(&N, g.xadj.data(), g.adj.data(), nullptr, nullptr,
                                        &sepsize, part.data());
  if (rc != 1) throw Error(RCHOL_ERR_INTERNAL, "METIS_ComputeVertexSeparator failed");
  part.resize(N);
  return part;
}

// c++/rchol/find_separator.cpp:23-56: rows of `par`, keeping the neighbours
// whose label equals the label of par[0].
Graph subgraph(const std::vector<int64_t> &par, const std::vector<int64_t> &label,
               const Graph &g) {
  Graph s;
  s.n = (int64_t)par.size();
  std::vector<int64_t> local(g.n, 0);
  for (size_t i = 0; i < par.size(); ++i) local[par[i]] = (int64_t)i;
  s.xadj.reserve(s.n + 1);
  s.xadj.push_back(0);
  int64_t lab = par.empty() ? -1 : label[par[0]];
  for (int64_t u : par) {
    for (int64_t j = g.xadj[u]; j < g.xadj[u + 1]; ++j)
      if (label[g.adj[j]] == lab) s.adj.push_back(local[g.adj[j]]);
    s.xadj.push_back((int64_t)s.adj.size());
  }
  return s;
}

// Order inside a leaf subdomain.  The C++ front end keeps the natural order
// (c++/rchol/find_separator.cpp:111-120); the MATLAB front end reorders every
// leaf with a fill-reducing ordering (matlab/rchol/find_separator.m:6, amd).
// Here: METIS nested dissection (METIS_NodeND) or a plain minimum-degree
// ordering (below).  Both change only the order inside leaves.
std::vector<int64_t> leaf_permutation(const Graph &g, int leaf_order) {
  const int64_t n = g.n;
  std::vector<int64_t> p(n);
  std::iota(p.begin(), p.end(), 0);
  if (leaf_order == RCHOL_LEAF_NATURAL || n <= 2) return p;
  if (leaf_order == RCHOL_LEAF_ND) {
    int64_t N = n;
    std::vector<int64_t> xadj(g.xadj), adj(g.adj), perm(n), iperm(n);
    if (adj.empty()) adj.push_back(0);
    int rc = METIS_NodeND(&N, xadj.data(), adj.data(), nullptr, nullptr, perm.data(), iperm.data());
    if (rc != 1) throw Error(RCHOL_ERR_INTERNAL, "METIS_NodeND failed");
    return perm;  // position i holds vertex perm[i]
  }
  // minimum degree: eliminate a vertex of least degree in the elimination
  // graph (ties: lowest index); its neighbours become a clique
  std::vector<std::vector<int64_t>> nb(n);
  std::set<std::pair<int64_t, int64_t>> q;
  for (int64_t i = 0; i < n; ++i) {
    for (int64_t j = g.xadj[i]; j < g.xadj[i + 1]; ++j)
      if (g.adj[j] != i) nb[i].push_back(g.adj[j]);
    std::sort(nb[i].begin(), nb[i].end());
    nb[i].erase(std::unique(nb[i].begin(), nb[i].end()), nb[i].end());
    q.insert({(int64_t)nb[i].size(), i});
  }
  int64_t k = 0;
  std::vector<int64_t> merged;
  while (!q.empty()) {
    const int64_t v = q.begin()->second;
    q.erase(q.begin());
    p[k++] = v;
    const std::vector<int64_t> N = std::move(nb[v]);
    nb[v].clear();
    for (int64_t u : N) {
      q.erase({(int64_t)nb[u].size(), u});
      merged.clear();
      std::set_union(nb[u].begin(), nb[u].end(), N.begin(), N.end(), std::back_inserter(merged));
      merged.erase(std::remove_if(merged.begin(), merged.end(), [&](int64_t x) { return x == u || x == v; }),
                   merged.end());
      nb[u].swap(merged);
      q.insert({(int64_t)nb[u].size(), u});
    }
  }
  return p;
}

// Number of partition segments below a node `levels` tree levels tall.
int64_t segments(int levels) { return ((int64_t)1 << levels) - 1; }

// c++/rchol/find_separator.cpp:109-163.  Writes the subtree's permutation
// (local ids, post-order) to p[0..g.n) and its partition sizes to
// val[0..segments(target-depth+1)).
//
// The METIS archive keeps its random-number state in process globals, so two
// threads calling it at once perturb each other's separators.  Subtrees are
// therefore ordered in forked child processes (while `forks` levels remain
// and the subgraph is large): the child inherits the subgraph, orders it with
// its own copy of METIS's state, writes the result into a shared anonymous
// mapping and exits without touching anything else.  Each METIS call sees
// exactly the subgraph the serial recursion would give it, so the ordering is
// identical to the serial one.
void dissect(Graph g, int depth, int target, int64_t *p, int64_t *val, int forks, bool last_in_root = false,
             int leaf_order = RCHOL_LEAF_NATURAL);

bool dissect_in_child(Graph &g, int depth, int target, int64_t *p, int64_t *val, int forks, int leaf_order,
                      pid_t *pid_out, int64_t **shm_out, size_t *shm_bytes) {
  const int64_t nseg = segments(target - depth + 1);
  size_t bytes = (size_t)(1 + g.n + nseg) * sizeof(int64_t);
  void *m = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_SHARED | MAP_ANONYMOUS, -1, 0);
  if (m == MAP_FAILED) return false;
  int64_t *shm = static_cast<int64_t *>(m);
  shm[0] = -1;  // status: 0 ok, 1 invalid argument, 2 other failure
  pid_t pid = fork();
  if (pid < 0) {
    munmap(m, bytes);
    return false;
  }
  if (pid == 0) {
    int64_t status = 2;
    try {
      dissect(std::move(g), depth, target, shm + 1, shm + 1 + g.n, forks, false, leaf_order);
      status = 0;
    } catch (const Error &e) {
      status = e.status == RCHOL_ERR_INVALID ? 1 : 2;
    } catch (...) {
      status = 2;
    }
    shm[0] = status;
    _exit(0);
  }
  *pid_out = pid;
  *shm_out = shm;
  *shm_bytes = bytes;
  return true;
}

void collect_child(pid_t pid, int64_t *shm, size_t bytes, int64_t n, int64_t nseg, int64_t *p,
                   int64_t *val) {
  int st = 0;
  while (waitpid(pid, &st, 0) < 0 && errno == EINTR) {
  }
  int64_t status = shm[0];
  if (status == 0) {
    std::memcpy(p, shm + 1, n * sizeof(int64_t));
    std::memcpy(val, shm + 1 + n, nseg * sizeof(int64_t));
  }
  munmap(shm, bytes);
  if (status == 1) throw Error(RCHOL_ERR_INVALID, "too many threads requested");
  if (status != 0) throw Error(RCHOL_ERR_INTERNAL, "nested-dissection worker process failed");
}

// last_in_root: the Python front end's variant, which puts the last vertex
// into the root separator (python/rchol_lap/find_separator.pyx:27-28).
void dissect(Graph g, int depth, int target, int64_t *p, int64_t *val, int forks, bool last_in_root,
             int leaf_order) {
  if (depth == target) {
    val[0] = g.n;
    const std::vector<int64_t> lp = leaf_permutation(g, leaf_order);
    std::copy(lp.begin(), lp.end(), p);
    return;
  }
  if (g.n <= 1) throw Error(RCHOL_ERR_INVALID, "too many threads requested");
  std::vector<int64_t> label = metis_separator(g);
  if (last_in_root && depth == 1) label[g.n - 1] = 2;
  std::vector<int64_t> l, r, s;
  for (int64_t i = 0; i < g.n; ++i) {
    if (label[i] == 0) l.push_back(i);
    else if (label[i] == 1) r.push_back(i);
    else s.push_back(i);
  }
  Graph gl = subgraph(l, label, g), gr = subgraph(r, label, g);
  g = Graph();  // release before recursing
  label.clear();
  label.shrink_to_fit();
  const int64_t nseg = segments(target - depth);  // per child
  std::vector<int64_t> pl(l.size()), pr(r.size()), vl(nseg), vr(nseg);
  pid_t pid = 0;
  int64_t *shm = nullptr;
  size_t shm_bytes = 0;
  bool forked = forks > 0 && gr.n >= 20000 &&
                dissect_in_child(gr, depth + 1, target, pr.data(), vr.data(), forks - 1, leaf_order, &pid, &shm,
                                 &shm_bytes);
  if (forked) {
    gr = Graph();  // the child owns its copy
    try {
      dissect(std::move(gl), depth + 1, target, pl.data(), vl.data(), forks - 1, false, leaf_order);
    } catch (...) {
      try {
        collect_child(pid, shm, shm_bytes, (int64_t)pr.size(), nseg, pr.data(), vr.data());
      } catch (...) {
      }
      throw;
    }
    collect_child(pid, shm, shm_bytes, (int64_t)pr.size(), nseg, pr.data(), vr.data());
  } else {
    dissect(std::move(gl), depth + 1, target, pl.data(), vl.data(), forks - 1, false, leaf_order);
    dissect(std::move(gr), depth + 1, target, pr.data(), vr.data(), forks - 1, false, leaf_order);
  }
  int64_t o = 0;
  for (int64_t x : vl) val[o++] = x;
  for (int64_t x : vr) val[o++] = x;
  val[o] = (int64_t)s.size();
  o = 0;
  for (int64_t x : pl) p[o++] = l[x];
  for (int64_t x : pr) p[o++] = r[x];
  for (int64_t x : s) p[o++] = x;
}

void build_nodes(rchol_tree_s &t) {
  t.nodes.clear();
  int64_t segs = (int64_t)t.part.size() - 1;
  int maxdepth = 1;
  std::function<void(int64_t, int64_t, int)> rec = [&](int64_t start, int64_t total, int depth) {
    maxdepth = std::max(maxdepth, depth);
    if (total == 1) {
      t.nodes.push_back(TreeNode{t.part[start], t.part[start + 1], depth, true});
      return;
    }
    int64_t h = (total - 1) / 2;
    rec(start, h, depth + 1);
    rec(start + h, h, depth + 1);
    t.nodes.push_back(TreeNode{t.part[start + total - 1], t.part[start + total], depth, false});
  };
  rec(0, segs, 1);
  t.depth = maxdepth;
}

}  // namespace

void validate_csr(int64_t n, const int64_t *rp, const int64_t *ci) {
  RCHOL_CHECK_ARG(n >= 1, "matrix must have at least one row");
  RCHOL_CHECK_ARG(n < (int64_t)INT32_MAX - 1, "matrix dimension must be below 2^31 - 1");
  RCHOL_CHECK_ARG(rp && ci, "null CSR array");
  RCHOL_CHECK_ARG(rp[0] == 0, "row_ptr[0] must be 0");
  for (int64_t i = 0; i < n; ++i) {
    RCHOL_CHECK_ARG(rp[i + 1] >= rp[i], "row_ptr must be nondecreasing");
    for (int64_t k = rp[i]; k < rp[i + 1]; ++k) {
      RCHOL_CHECK_ARG(ci[k] >= 0 && ci[k] < n, "column index out of range");
      RCHOL_CHECK_ARG(k == rp[i] || ci[k] > ci[k - 1], "column indices must be strictly increasing within a row");
    }
  }
}

rchol_tree_s *build_tree(int64_t n, const int64_t *rp, const int64_t *ci, int threads, bool last_in_root,
                         int leaf_order) {
  RCHOL_CHECK_ARG(threads > 0, "thread number should be positive");
  RCHOL_CHECK_ARG((threads & (threads - 1)) == 0, "thread number should be a power of 2");
  validate_csr(n, rp, ci);
  auto t = new rchol_tree_s();
  try {
    t->n = n;
    t->threads = threads;
    int target = 1;
    while ((1 << (target - 1)) < threads) ++target;
    std::vector<int64_t> val;
    if (target == 1 && leaf_order == RCHOL_LEAF_NATURAL) {
      t->perm.resize(n);
      std::iota(t->perm.begin(), t->perm.end(), 0);
      val.assign(1, n);
    } else {
      Graph g;
      g.n = n;
      g.xadj.resize(n + 1);
      g.xadj[0] = 0;
      for (int64_t i = 0; i < n; ++i) {
        int64_t c = 0;
        for (int64_t k = rp[i]; k < rp[i + 1]; ++k) c += (ci[k] != i);
        g.xadj[i + 1] = g.xadj[i] + c;
      }
      g.adj.resize(g.xadj[n]);
      parallel_for(n, [&](int64_t a, int64_t b) {
        for (int64_t i = a; i < b; ++i) {
          int64_t o = g.xadj[i];
          for (int64_t k = rp[i]; k < rp[i + 1]; ++k)
            if (ci[k] != i) g.adj[o++] = ci[k];
        }
      }, 1 << 16);
      int forks = 0;
      while ((1 << forks) < host_threads()) ++forks;
      if (const char *e = getenv("RCHOL_ORDER_FORK_LEVELS")) forks = atoi(e);
      t->perm.resize(n);
      val.resize(segments(target));
      dissect(std::move(g), 1, target, t->perm.data(), val.data(), forks, last_in_root, leaf_order);
    }
    t->part.assign(1, 0);
    for (int64_t x : val) t->part.push_back(t->part.back() + x);
    t->part.back() += 1;
    build_nodes(*t);
    return t;
  } catch (...) {
    delete t;
    throw;
  }
}

rchol_tree_s *tree_from_partition(int64_t n, const int64_t *perm, const int64_t *part,
                                  int64_t nparts) {
  RCHOL_CHECK_ARG(n >= 1 && perm && part, "invalid ordering arguments");
  RCHOL_CHECK_ARG(nparts >= 2 && (nparts & (nparts - 1)) == 0,
                  "partition length must be twice a power of two");
  RCHOL_CHECK_ARG(part[0] == 0 && part[nparts - 1] == n + 1,
                  "partition must start at 0 and end at n+1 (ground vertex included)");
  for (int64_t i = 0; i + 1 < nparts; ++i)
    RCHOL_CHECK_ARG(part[i + 1] >= part[i], "partition must be nondecreasing");
  std::vector<char> seen(n, 0);
  for (int64_t i = 0; i < n; ++i) {
    RCHOL_CHECK_ARG(perm[i] >= 0 && perm[i] < n && !seen[perm[i]], "perm is not a permutation");
    seen[perm[i]] = 1;
  }
  auto t = new rchol_tree_s();
  t->n = n;
  t->threads = (int)(nparts / 2);
  t->perm.assign(perm, perm + n);
  t->part.assign(part, part + nparts);
  build_nodes(*t);
  return t;
}

// Many independent systems as one block-diagonal matrix: every system is
// ordered on its own (the same nested dissection as build_tree, `threads`
// leaves each), and the per-system trees become the subtrees of one complete
// binary tree whose upper separators are empty.  The system count is padded
// to a power of two with empty systems, so the union has the post-order
// result_idx layout of a single ordering with nsys_pad * threads leaves.  The
// ground vertex sits in the (otherwise empty) root separator; no elimination
// creates an edge between two systems, so G is block diagonal.  Each system
// keeps its rows [sys_ptr[s], sys_ptr[s+1]) under the permutation.
rchol_tree_s *build_tree_batch(int64_t nsys, const int64_t *sys_ptr, int64_t n, const int64_t *rp,
                               const int64_t *ci, int threads) {
  RCHOL_CHECK_ARG(nsys >= 1 && sys_ptr, "need at least one system");
  RCHOL_CHECK_ARG(threads > 0 && (threads & (threads - 1)) == 0, "thread number should be a power of 2");
  RCHOL_CHECK_ARG(sys_ptr[0] == 0 && sys_ptr[nsys] == n, "system offsets must run from 0 to n");
  for (int64_t s = 0; s < nsys; ++s)
    RCHOL_CHECK_ARG(sys_ptr[s + 1] > sys_ptr[s], "every system needs at least one row");
  validate_csr(n, rp, ci);
  for (int64_t s = 0; s < nsys; ++s)
    for (int64_t i = sys_ptr[s]; i < sys_ptr[s + 1]; ++i)
      for (int64_t q = rp[i]; q < rp[i + 1]; ++q)
        RCHOL_CHECK_ARG(ci[q] >= sys_ptr[s] && ci[q] < sys_ptr[s + 1],
                        "the matrix must be block diagonal over the systems");
  int64_t pad = 1;
  while (pad < nsys) pad *= 2;
  const int64_t segs_sys = 2 * (int64_t)threads - 1;
  std::vector<std::vector<int64_t>> part_sys(nsys);  // segment sizes per system
  auto t = new rchol_tree_s();
  try {
    t->n = n;
    t->perm.resize(n);
    for (int64_t s = 0; s < nsys; ++s) {
      const int64_t b = sys_ptr[s], ns = sys_ptr[s + 1] - b;
      std::vector<int64_t> lrp(ns + 1), lci;
      lci.reserve(rp[sys_ptr[s + 1]] - rp[b]);
      for (int64_t i = 0; i < ns; ++i) {
        for (int64_t q = rp[b + i]; q < rp[b + i + 1]; ++q) lci.push_back(ci[q] - b);
        lrp[i + 1] = (int64_t)lci.size();
      }
      std::unique_ptr<rchol_tree_s> ts(build_tree(ns, lrp.data(), lci.data(), threads));
      for (int64_t i = 0; i < ns; ++i) t->perm[b + i] = ts->perm[i] + b;
      std::vector<int64_t> &sz = part_sys[s];
      sz.resize(segs_sys);
      for (int64_t j = 0; j < segs_sys; ++j) sz[j] = ts->part[j + 1] - ts->part[j];
      sz.back() -= 1;  // the system's own ground slot; the union has one ground
    }
    // post-order of the complete tree over padded systems
    std::vector<int64_t> sizes;
    std::function<void(int64_t, int64_t)> rec = [&](int64_t s0, int64_t cnt) {
      if (cnt == 1) {
        if (s0 < nsys) sizes.insert(sizes.end(), part_sys[s0].begin(), part_sys[s0].end());
        else sizes.insert(sizes.end(), segs_sys, 0);
        return;
      }
      rec(s0, cnt / 2);
      rec(s0 + cnt / 2, cnt / 2);
      sizes.push_back(0);  // empty separator joining the two halves
    };
    rec(0, pad);
    t->threads = (int)(pad * threads);
    t->part.assign(1, 0);
    for (int64_t x : sizes) t->part.push_back(t->part.back() + x);
    t->part.back() += 1;  // ground vertex in the root separator
    build_nodes(*t);
    return t;
  } catch (...) {
    delete t;
    throw;
  }
}

// c++/util/util.cpp:16-49: B = A(p,p) with each row's columns sorted.
HostCsr reorder(int64_t n, const int64_t *rp, const int64_t *ci, const double *v,
                const std::vector<int64_t> &perm, std::vector<int64_t> *srcpos) {
  std::vector<int64_t> inv(n);
  for (int64_t i = 0; i < n; ++i) inv[perm[i]] = i;
  HostCsr B;
  B.n = n;
  B.rp.assign(n + 1, 0);
  for (int64_t i = 0; i < n; ++i) B.rp[i + 1] = B.rp[i] + (rp[perm[i] + 1] - rp[perm[i]]);
  B.ci.resize(B.rp[n]);
  B.v.resize(B.rp[n]);
  if (srcpos) srcpos->resize(B.rp[n]);
  parallel_for(n, [&](int64_t a, int64_t b) {
    std::vector<std::pair<int64_t, int64_t>> row;  // (new column, source position)
    for (int64_t i = a; i < b; ++i) {
      int64_t o = perm[i];
      row.clear();
      for (int64_t k = rp[o]; k < rp[o + 1]; ++k) row.emplace_back(inv[ci[k]], k);
      std::sort(row.begin(), row.end(),
                [](const std::pair<int64_t, int64_t> &x, const std::pair<int64_t, int64_t> &y) {
                  return x.first < y.first;
                });
      int64_t w = B.rp[i];
      for (auto &e : row) {
        B.ci[w] = e.first;
        B.v[w] = v ? v[e.second] : 0.0;
        if (srcpos) (*srcpos)[w] = e.second;
        ++w;
      }
    }
  }, 1 << 14);
  return B;
}

// c++/util/util.hpp:60-142 and :85-91: the upper triangle of A plus a ground
// vertex n that takes the excess of every row, all values negated.
HostCsr extend_laplacian(const HostCsr &A) {
  int64_t n = A.n;
  std::vector<double> rowsum(n);
  std::vector<int64_t> cnt(n + 1, 0);
  parallel_for(n, [&](int64_t a, int64_t b) {
    for (int64_t r = a; r < b; ++r) {
      double s = 0.0;
      int64_t c = 0;
      for (int64_t k = A.rp[r]; k < A.rp[r + 1]; ++k) {
        s += A.v[k];
        c += (A.ci[k] >= r);
      }
      rowsum[r] = s;
      cnt[r] = c + (std::abs(s) > 1e-09 ? 1 : 0);
    }
  }, 1 << 14);
  double overall = 0.0;
  for (int64_t r = 0; r < n; ++r) overall -= rowsum[r];
  cnt[n] = std::abs(overall) > 1e-09 ? 1 : 0;
  HostCsr L;
  L.n = n + 1;
  L.rp.assign(n + 2, 0);
  for (int64_t r = 0; r <= n; ++r) L.rp[r + 1] = L.rp[r] + cnt[r];
  L.ci.resize(L.rp[n + 1]);
  L.v.resize(L.rp[n + 1]);
  parallel_for(n, [&](int64_t a, int64_t b) {
    for (int64_t r = a; r < b; ++r) {
      int64_t w = L.rp[r];
      for (int64_t k = A.rp[r]; k < A.rp[r + 1]; ++k)
        if (A.ci[k] >= r) {
          L.ci[w] = A.ci[k];
          L.v[w] = -A.v[k];
          ++w;
        }
      if (std::abs(rowsum[r]) > 1e-09) {
        L.ci[w] = n;
        L.v[w] = rowsum[r];  // -(-sum)
      }
    }
  }, 1 << 14);
  if (cnt[n]) {
    L.ci[L.rp[n]] = n;
    L.v[L.rp[n]] = overall;  // -(-overall)
  }
  return L;
}

std::vector<TreeNode> trivial_nodes(int64_t n) {
  return std::vector<TreeNode>{TreeNode{0, n + 1, 1, true}};
}

}  // namespace rchol
