// Host-side helpers shared by the C ABI and the device code drivers.
#pragma once

#include <functional>
#include <vector>

#include "common.hpp"

namespace rchol {

int host_threads();
void parallel_for(int64_t n, const std::function<void(int64_t, int64_t)> &body, int64_t grain);

void validate_csr(int64_t n, const int64_t *rp, const int64_t *ci);
// Order inside the leaf subdomains (see leaf_permutation in host.cpp).
enum { RCHOL_LEAF_NATURAL = 0, RCHOL_LEAF_ND = 1, RCHOL_LEAF_MD = 2 };

// last_in_root: the Python front end's ordering (last vertex forced into the
// root separator); false: the C++ front end's.
rchol_tree_s *build_tree(int64_t n, const int64_t *rp, const int64_t *ci, int threads,
                         bool last_in_root = false, int leaf_order = RCHOL_LEAF_NATURAL);
rchol_tree_s *tree_from_partition(int64_t n, const int64_t *perm, const int64_t *part,
                                  int64_t nparts);
rchol_tree_s *build_tree_batch(int64_t nsys, const int64_t *sys_ptr, int64_t n, const int64_t *rp,
                               const int64_t *ci, int threads);
// B = A(perm, perm); srcpos[q] = position in A of B's entry q.
HostCsr reorder(int64_t n, const int64_t *rp, const int64_t *ci, const double *v,
                const std::vector<int64_t> &perm, std::vector<int64_t> *srcpos = nullptr);
HostCsr extend_laplacian(const HostCsr &A);
std::vector<TreeNode> trivial_nodes(int64_t n);

// Device drivers (factor.cu, solve.cu).
void gpu_factor(const HostCsr &ext, const std::vector<TreeNode> &nodes, uint64_t seed,
                rchol_factor_s &F, cudaStream_t s);
void finish_factor(rchol_factor_s &F, cudaStream_t s);  // transpose, FP32 copies, plan
void build_plan(rchol_factor_s &F, cudaStream_t s);

}  // namespace rchol
