/* Declarations standing in for METIS (not installed here).  The reference's porder.hpp
   includes metis.h for its METIS order only; the GRO order built from it never calls
   METIS, and ref_metis_stub.cpp defines the one function so the program links. */
#ifndef ATC_SHIM_METIS_H_
#define ATC_SHIM_METIS_H_
#include <stdint.h>
typedef int32_t idx_t;
typedef float real_t;
#define METIS_OK 1
#define METIS_NOPTIONS 40
int METIS_PartGraphRecursive(idx_t* nvtxs, idx_t* ncon, idx_t* xadj, idx_t* adjncy, idx_t* vwgt, idx_t* vsize,
                             idx_t* adjwgt, idx_t* nparts, real_t* tpwgts, real_t* ubvec, idx_t* options,
                             idx_t* edgecut, idx_t* part);
int METIS_SetDefaultOptions(idx_t* options);
#endif
