// The nested-dissection tree of a factor given without one.
//
// A G made elsewhere -- by the reference's own rchol() (c++/rchol/rchol_parallel.cpp:37-92),
// or copied, so that the library no longer holds the tree it was factored
// with -- still has the structure of its ordering: in a nested-dissection
// order every subtree is a contiguous range of rows whose entries stay inside
// the range, with the left subtree first, then the right one, then the
// separator.  This file recovers such a tree from G's nonzero pattern alone,
// so that the solves run the independent subtrees in parallel instead of as
// one chain.
//
// For a range [b, e) whose rows only read columns in [b, e), a split point m
// gives a left part [b, m) (self-contained, G being lower triangular), a
// right part [m, s(m)) with s(m) = the first row >= m that reads a column
// below m, and a separator [s(m), e).  Every split is exact by construction
// (no row of the right part reads the left one), so the tree is valid for
// any G; the heuristic only decides how much parallelism is found.  The
// split taken maximises min(m - b, s(m) - m); ranges below kInferMinRows, or
// whose best split leaves a part under 1/16 of the range, stay leaves.

#pragma once

#include <algorithm>
#include <cstdint>
#include <functional>
#include <queue>
#include <vector>

#include "common.hpp"

namespace rchol {

constexpr int64_t kInferMinRows = 256;
constexpr int kInferMaxDepth = 24;

// gt_rp / gt_ci: CSR of G^T (row j = column j of G, entries at rows >= j).
inline std::vector<TreeNode> infer_factor_tree(int64_t n, const int64_t *gt_rp, const int64_t *gt_ci) {
  // minc[i]: the smallest column row i of G reads (i itself if none)
  std::vector<int64_t> minc(n);
  for (int64_t i = 0; i < n; ++i) minc[i] = i;
  for (int64_t j = 0; j < n; ++j)
    for (int64_t q = gt_rp[j]; q < gt_rp[j + 1]; ++q) {
      const int64_t i = gt_ci[q];
      if (i > j && j < minc[i]) minc[i] = j;
    }
  std::vector<TreeNode> nodes;
  std::vector<int64_t> start, rows;  // rows of [b, e) bucketed by minc
  std::function<void(int64_t, int64_t, int)> rec = [&](int64_t b, int64_t e, int depth) {
    const int64_t len = e - b;
    int64_t best_m = -1, best_s = -1, best = 0;
    if (len >= kInferMinRows && depth < kInferMaxDepth) {
      // s(m) for all m in (b, e): rows i with minc[i] < m <= i block m; a
      // min-heap of the blocking rows (entered at m = minc[i] + 1, expired
      // once m > i) gives the first one
      start.assign(len + 1, 0);
      for (int64_t i = b; i < e; ++i)
        if (minc[i] < i) ++start[minc[i] - b + 1];
      for (int64_t k = 0; k < len; ++k) start[k + 1] += start[k];
      rows.assign(start[len], 0);
      {
        std::vector<int64_t> fill(start.begin(), start.end() - 1);
        for (int64_t i = b; i < e; ++i)
          if (minc[i] < i) rows[fill[minc[i] - b]++] = i;
      }
      std::priority_queue<int64_t, std::vector<int64_t>, std::greater<int64_t>> heap;
      for (int64_t m = b + 1; m < e; ++m) {
        for (int64_t k = start[m - 1 - b]; k < start[m - b]; ++k) heap.push(rows[k]);  // minc = m - 1
        while (!heap.empty() && heap.top() < m) heap.pop();
        const int64_t s = heap.empty() ? e : heap.top();
        const int64_t score = std::min(m - b, s - m);
        if (score > best) {
          best = score;
          best_m = m;
          best_s = s;
        }
      }
    }
    if (best_m < 0 || best * 16 < len) {
      nodes.push_back(TreeNode{b, e, depth, true});
      return;
    }
    rec(b, best_m, depth + 1);
    rec(best_m, best_s, depth + 1);
    nodes.push_back(TreeNode{best_s, e, depth, false});
  };
  rec(0, n, 1);
  return nodes;
}

}  // namespace rchol
