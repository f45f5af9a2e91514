/* Minimal METIS 5 declarations for the oracle build of the reference.
 * The METIS archive shipped with the CUDA toolkit (libmetis_static.a) is
 * built with 64-bit idx_t; no metis.h ships with it.  Test infrastructure
 * only. */
#pragma once
#include <stdint.h>
typedef int64_t idx_t;
#ifdef __cplusplus
extern "C" {
#endif
int METIS_ComputeVertexSeparator(idx_t *nvtxs, idx_t *xadj, idx_t *adjncy,
                                 idx_t *vwgt, idx_t *options, idx_t *sepsize,
                                 idx_t *part);
int METIS_NodeND(idx_t *nvtxs, idx_t *xadj, idx_t *adjncy, idx_t *vwgt, idx_t *options,
                 idx_t *perm, idx_t *iperm);
#ifdef __cplusplus
}
#endif
