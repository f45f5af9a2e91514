/*
 * rchol_gpu.h -- C ABI of the GB300 implementation of rchol's
 * preconditioned-solve path: nested-dissection ordering on the host,
 * randomized Cholesky factorization and preconditioned conjugate gradients on
 * one GPU.
 *
 * Every entry point takes plain pointers and sizes.  Index arrays are
 * int64_t (the reference's size_t, c++/sparse.hpp:26-30); values are double.
 * Matrices are 0-based CSR with sorted column indices and an explicit
 * diagonal.  Functions return RCHOL_OK (0) or an RCHOL_ERR_* status and leave
 * a message for rchol_gpu_last_error() (thread-local).  The reference throws
 * std::invalid_argument instead (c++/rchol/rchol_parallel.cpp:39-43,
 * c++/rchol/find_separator.cpp:125); include/rchol_gb300.hpp rethrows.
 *
 * Handles own their memory: each *_create / *_build has a matching *_destroy.
 * `stream` is a cudaStream_t passed as void* (NULL = the legacy stream).
 * Pointers named d_* are device pointers; all others are host pointers.
 */
#ifndef RCHOL_GPU_H
#define RCHOL_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
  RCHOL_OK = 0,
  RCHOL_ERR_INVALID = 1,  /* bad argument (reference: std::invalid_argument) */
  RCHOL_ERR_CUDA = 2,     /* a CUDA runtime call failed */
  RCHOL_ERR_SINGULAR = 3, /* a pivot of the factorization was not positive */
  RCHOL_ERR_NOMEM = 4,    /* device or host allocation failed */
  RCHOL_ERR_TIMEOUT = 5,  /* a bounded device-side wait gave up */
  RCHOL_ERR_INTERNAL = 6
};

/* Precision in which G is stored and applied by the triangular solves.  The
 * factorization's accumulation and the outer PCG are FP64 either way. */
enum { RCHOL_PREC_FP64 = 0, RCHOL_PREC_FP32 = 1 };

typedef struct rchol_tree_s *rchol_tree_t;     /* ordering + separator tree (host) */
typedef struct rchol_matrix_s *rchol_matrix_t; /* SDDM matrix resident on the GPU  */
typedef struct rchol_factor_s *rchol_factor_t; /* factor G resident on the GPU     */

const char *rchol_gpu_last_error(void);
const char *rchol_gpu_version(void);
/* Number of GPU kernels the solve entry points have launched so far in this
 * process (SpMV, triangular solves, PCG); for launch accounting. */
int64_t rchol_gpu_launch_count(void);

/* ---- ordering (host) ------------------------------------------------------
 * Nested dissection to depth log2(threads)+1 by recursive METIS vertex
 * separators.  Replaces remove_diagonal + find_separator + the result_idx
 * prefix of c++/rchol/rchol_parallel.cpp:9-70 (find_separator.cpp:109-163).
 * `threads` (the reference's thread count) is the number of leaf subdomains
 * and must be a power of two.  threads == 1 gives the identity order and one
 * subdomain, which is what the sequential rchol(A, G) uses
 * (c++/rchol/rchol.cpp:26).  perm is new->old; part is result_idx (2*threads
 * entries, the last one counting the ground vertex). */
int rchol_gpu_tree_build(int64_t n, const int64_t *row_ptr, const int64_t *col_idx,
                         int threads, rchol_tree_t *out);
/* The same with ordering flags.  RCHOL_ORDER_LAST_IN_ROOT reproduces the
 * Python front end's ordering, which forces the last vertex into the root
 * separator (python/rchol_lap/find_separator.pyx:27-28, called from
 * python/rchol/rchol.py:31-33); without it the ordering is the C++ front
 * end's (c++/rchol/find_separator.cpp). */
#define RCHOL_ORDER_LAST_IN_ROOT 1
/* Fill-reducing order inside every leaf subdomain instead of the natural one
 * (the MATLAB front end orders leaves with amd, matlab/rchol/find_separator.m:6):
 * METIS nested dissection, or a minimum-degree ordering (for small leaves). */
#define RCHOL_ORDER_LEAF_ND 2
#define RCHOL_ORDER_LEAF_MD 4
int rchol_gpu_tree_build_ex(int64_t n, const int64_t *row_ptr, const int64_t *col_idx,
                            int threads, int flags, rchol_tree_t *out);
/* Many independent systems at once (no counterpart in the reference, which
 * orders one matrix per call): the matrix is block diagonal with system s on
 * rows [sys_ptr[s], sys_ptr[s+1]).  Each system is ordered like
 * rchol_gpu_tree_build with `threads` leaves and keeps its row range under
 * the permutation; the systems' trees hang below empty separators of one
 * tree, so the factor of the whole matrix is block diagonal. */
int rchol_gpu_tree_build_batch(int64_t nsys, const int64_t *sys_ptr, int64_t n,
                               const int64_t *row_ptr, const int64_t *col_idx, int threads,
                               rchol_tree_t *out);
/* Reuse a stored ordering (python/rchol/rchol.py:24-34). */
int rchol_gpu_tree_from_partition(int64_t n, const int64_t *perm, const int64_t *part,
                                  int64_t nparts, rchol_tree_t *out);
int64_t rchol_gpu_tree_size(rchol_tree_t tree);      /* n */
int64_t rchol_gpu_tree_num_parts(rchol_tree_t tree); /* length of part */
int rchol_gpu_tree_get(rchol_tree_t tree, int64_t *perm, int64_t *part);
void rchol_gpu_tree_destroy(rchol_tree_t tree);

/* B = A(perm, perm) with sorted rows, on the host (c++/util/util.cpp:16-49,
 * used by c++/ex_laplace_parallel.cpp:38).  B has A's nnz; the out arrays
 * must hold n+1, nnz and nnz entries. */
int rchol_gpu_reorder(int64_t n, const int64_t *row_ptr, const int64_t *col_idx,
                      const double *val, const int64_t *perm, int64_t *out_row_ptr,
                      int64_t *out_col_idx, double *out_val);

/* ---- matrices --------------------------------------------------------------
 * Upload an SDDM matrix.  With a tree, the matrix is stored permuted, A(p,p)
 * (c++/util/util.cpp:16-49), which is the system pcg() solves in the
 * reference's parallel example (c++/ex_laplace_parallel.cpp:38-39). */
int rchol_gpu_matrix_create(int64_t n, const int64_t *row_ptr, const int64_t *col_idx,
                            const double *val, rchol_tree_t tree, rchol_matrix_t *out);
int64_t rchol_gpu_matrix_size(rchol_matrix_t A);
int64_t rchol_gpu_matrix_nnz(rchol_matrix_t A);
/* Replace the values (same sparsity pattern, same ordering). */
int rchol_gpu_matrix_set_values(rchol_matrix_t A, const double *val);
void rchol_gpu_matrix_destroy(rchol_matrix_t A);

/* ---- factorization ---------------------------------------------------------
 * Randomized Cholesky of the extended Laplacian of A on the GPU.  Replaces
 * rchol_lap (c++/rchol_lap/rchol_lap.cpp:138-150, :187-387).  A must have been
 * created with the same tree.  The sampler is a Philox4x32-10 stream keyed by
 * (seed, vertex, sample), so the result depends only on the ordering and the
 * seed. */
int rchol_gpu_factor(rchol_matrix_t A, rchol_tree_t tree, uint64_t seed, int precision,
                     rchol_factor_t *out);
/* Load a factor computed elsewhere (e.g. by the reference): CSR of G^T with
 * the diagonal first in each row, as rchol() returns it.  Without `tree`, the
 * nested-dissection structure is read off G's nonzero pattern (contiguous
 * ranges whose rows only read inside them), so independent subtrees are still
 * solved in parallel. */
int rchol_gpu_factor_from_host(int64_t n, const int64_t *row_ptr, const int64_t *col_idx,
                               const double *val, rchol_tree_t tree, int precision,
                               rchol_factor_t *out);
int64_t rchol_gpu_factor_nnz(rchol_factor_t G);
int rchol_gpu_factor_precision(rchol_factor_t G);
/* Copy G back as CSR of G^T (row_ptr: n+1, col_idx/val: nnz). */
int rchol_gpu_factor_export(rchol_factor_t G, int64_t *row_ptr, int64_t *col_idx, double *val);
/* Pivots d of the factorization (length n), G = L sqrt(D). */
int rchol_gpu_factor_pivots(rchol_factor_t G, double *d);
/* Shape of the triangular-solve plan of the forward (transpose = 0) or
 * backward solve: stages (kernel pairs in sequence), pieces, and the
 * sequential 32-row block steps on the critical path.  No counterpart in
 * the reference. */
int rchol_gpu_factor_plan_info(rchol_factor_t G, int transpose, int64_t *stages, int64_t *pieces, int64_t *steps);
/* Autotuning of the solves on this factor: times the preconditioner with
 * alternative launch choices (L2 prefetch distance and ring depth of the
 * pipeline format, warps per thread block and prefetch of the warp format)
 * and keeps the fastest for all later solves with G.  ms_before / ms_after:
 * preconditioner time with the choices on entry / chosen; knobs (4 ints, may
 * be NULL): pipeline prefetch, pipeline ring, warp-format warps per block,
 * warp-format prefetch.  Allocates scratch, synchronises the device.  No
 * counterpart in the reference. */
int rchol_gpu_factor_tune(rchol_factor_t G, double *ms_before, double *ms_after, int *knobs);
/* Wall time (seconds) of the set-up phases that made G: the elimination
 * kernels (0 for rchol_gpu_factor_from_host), the assembly of G (transpose,
 * row sort, FP32 copies) and the triangular-solve plan.  No counterpart in
 * the reference. */
int rchol_gpu_factor_setup_times(rchol_factor_t G, double *eliminate_s, double *assemble_s, double *plan_s);
/* Level-schedule depth of the forward and backward solves. */
int rchol_gpu_factor_levels(rchol_factor_t G, int64_t *fwd_levels, int64_t *bwd_levels);
void rchol_gpu_factor_destroy(rchol_factor_t G);

/* ---- solves ----------------------------------------------------------------
 * Preconditioned CG with M^-1 = (G G^T)^-1 following c++/util/pcg.cpp:57-127
 * (alpha from p.r, beta from (r.z)/(r_prev.z_prev), x0 = 0, stop when
 * ||r|| <= tol*||b|| or after maxit iterations; relres = ||Ax-b||/||b||).
 * b and x hold nrhs right-hand sides as a row-major n x nrhs block (the nrhs
 * values of row i are contiguous); every right-hand side gets its own alpha,
 * beta and stopping test and one traversal of A and G serves all of them.  relres and itr
 * have nrhs entries.  The d_ variant takes device pointers and runs on
 * `stream`; the host variant copies b in and x out itself. */
int rchol_gpu_pcg(rchol_matrix_t A, rchol_factor_t G, const double *b, double *x,
                  int64_t nrhs, double tol, int maxit, double *relres, int *itr);
int rchol_gpu_pcg_d(rchol_matrix_t A, rchol_factor_t G, const double *d_b, double *d_x,
                    int64_t nrhs, double tol, int maxit, double *relres, int *itr,
                    void *stream);
/* Independent PCG solves (c++/util/pcg.cpp:57-127 per system) of the
 * diagonal blocks of A, system s on the (permuted) rows [sys_ptr[s],
 * sys_ptr[s+1]), with a block-diagonal G (a factor of a matrix ordered by
 * rchol_gpu_tree_build_batch).  Every system has its own scalars, stopping
 * test and iteration count; relres and itr have nsys entries.  One SpMV and
 * one preconditioner apply per iteration serve all systems.  No counterpart
 * in the reference. */
int rchol_gpu_pcg_batch(rchol_matrix_t A, rchol_factor_t G, int64_t nsys, const int64_t *sys_ptr,
                        const double *b, double *x, double tol, int maxit, double *relres,
                        int *itr);
int rchol_gpu_pcg_batch_d(rchol_matrix_t A, rchol_factor_t G, int64_t nsys,
                          const int64_t *sys_ptr, const double *d_b, double *d_x, double tol,
                          int maxit, double *relres, int *itr, void *stream);
/* z = (G G^T)^-1 r (c++/util/pcg.cpp:141-159); device pointers. */
int rchol_gpu_precond_d(rchol_factor_t G, const double *d_r, double *d_z, int64_t nrhs,
                        void *stream);
/* z = (G G^T)^-1 r for one right-hand side without allocating any memory.
 * No counterpart in the reference.  For callers that cannot allocate device
 * memory at solve time (a memory budget fixed at start-up, allocator-free
 * real-time loops, hosts that own all device memory): the two scratch vectors
 * live in a fixed 16 MiB device array inside the library, held on every GPU
 * that loads it until the process exits, so n is limited to 1,048,576 for an
 * FP64 factor and 2,097,152 for an FP32 one (larger n: RCHOL_ERR_INVALID).
 * The first call on a device looks up the array's device address (make it
 * before any stream capture); later calls on a stream that is not capturing
 * look it up again, so a device reset leaves no stale address.  All calls
 * share the array: calls that overlap on the GPU race.  Device pointers. */
int rchol_gpu_precond_noalloc_d(rchol_factor_t G, const double *d_r, double *d_z, void *stream);
/* Forward (y = G^-1 r) or backward (z = G^-T y) solve alone; device pointers. */
int rchol_gpu_trsv_d(rchol_factor_t G, int transpose, const double *d_in, double *d_out,
                     int64_t nrhs, void *stream);
/* y = A x (c++/util/pcg.cpp:130-138); device pointers. */
int rchol_gpu_spmv_d(rchol_matrix_t A, const double *d_x, double *d_y, int64_t nrhs,
                     void *stream);
/* Status of the triangular-solve kernels since the last check (no reference
 * counterpart: the reference's solves are host loops).  Their waits for
 * record copies are bounded; a wait that gives up marks a device-wide flag
 * and the kernel finishes without using the data.  This call synchronizes
 * `stream`, reads and clears the flag, and returns RCHOL_OK or
 * RCHOL_ERR_TIMEOUT (a wait gave up: the solve's output is not valid).  The
 * PCG entry points check it before returning; after
 * rchol_gpu_precond_d / _noalloc_d / rchol_gpu_trsv_d the caller does.  The
 * flag is shared by all streams of the device. */
int rchol_gpu_solve_status(void *stream);
/* Runs one bounded wait that nothing completes (`polls` polls of an mbarrier
 * no thread arrives at) and returns rchol_gpu_solve_status: RCHOL_ERR_TIMEOUT
 * shows the timeout path works on this device, without a fault. */
int rchol_gpu_wait_selftest(uint32_t polls, void *stream);

/* ---- differentiation ---------------------------------------------------------
 * No counterpart in the reference (its Python/MATLAB front ends are not
 * differentiable).  For A(w) = sum_e w_e (u_i - u_j)(u_i - u_j)^T + diag(s),
 * x = A^-1 b and the adjoint lambda = A^-1 dL/dx (the same G serves both
 * solves because A is symmetric):
 *   grad[e] = dL/dw_e = -(lambda_i - lambda_j) * (x_i - x_j)   for e = (ei[e], ej[e]).
 * Device pointers; indices refer to the vectors as passed. */
int rchol_gpu_edge_grad_d(int64_t nedges, const int64_t *d_ei, const int64_t *d_ej,
                          const double *d_lambda, const double *d_x, double *d_grad, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RCHOL_GPU_H */
