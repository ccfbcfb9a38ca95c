// Single-rank stand-in for the two METIS 5 routines the reference's partitioner calls (TEST
// INFRASTRUCTURE ONLY).  With one part there is nothing to partition: METIS_PartGraphKway puts
// every element in part 0 and METIS_MeshToDual returns a graph without edges (the reference uses
// the dual graph only to find inter-part and periodic interfaces, which one part without
// periodic boundaries does not have).  Implemented in oracle/refpin/refpin_runtime.cpp.
#pragma once
#include <stdint.h>
typedef int32_t idx_t;
typedef float real_t;
#define METIS_OK 1
#define METIS_ERROR -4
#define METIS_NOPTIONS 40
#define METIS_OPTION_NUMBERING 17
int METIS_MeshToDual(idx_t* ne, idx_t* nn, idx_t* eptr, idx_t* eind, idx_t* ncommon, idx_t* numflag, idx_t** xadj,
                     idx_t** adjncy);
int METIS_PartGraphKway(idx_t* nvtxs, idx_t* ncon, idx_t* xadj, idx_t* adjncy, idx_t* vwgt, idx_t* vsize,
                        idx_t* adjwgt, idx_t* nparts, real_t* tpwgts, real_t* ubvec, idx_t* options, idx_t* edgecut,
                        idx_t* part);
int METIS_Free(void* ptr);
