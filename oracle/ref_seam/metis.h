/*
 * metis.h -- link seam for building the reference's own sources without METIS.
 *
 * TEST INFRASTRUCTURE ONLY.  The reference partitions with
 * METIS_PartGraphKway (src/decomp/domain_decomp.h:23-58, METIS 5.1.0 per
 * spack.yaml:5), which is not installed here.  This header declares the one
 * METIS entry point the reference calls with METIS's default 32-bit index
 * type; ref_shim.cpp defines it to return a partition vector injected by the
 * test harness, so the reference build and the CUDA path see the same
 * partition.
 */
#pragma once
#include <stdint.h>

typedef int32_t idx_t;
typedef float real_t;

#define METIS_OK 1
#define METIS_ERROR_INPUT (-2)

#ifdef __cplusplus
extern "C" {
#endif
int METIS_PartGraphKway(idx_t* nvtxs, idx_t* ncon, idx_t* xadj, idx_t* adjncy,
                        idx_t* vwgt, idx_t* vsize, idx_t* adjwgt, idx_t* nparts,
                        real_t* tpwgts, real_t* ubvec, idx_t* options, idx_t* objval,
                        idx_t* part);
#ifdef __cplusplus
}
#endif
