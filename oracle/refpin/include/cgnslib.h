// Stand-in for the CGNS library interface the reference's -cgns reader names (TEST
// INFRASTRUCTURE ONLY).  C linkage, as the CGNS library has.  CGNS input is not exercised: cg_open fails with an error message, so
// a run given -cgns stops in the reference's own error handler.  Implemented in
// oracle/refpin/refpin_runtime.cpp.
#pragma once
#include <stdint.h>
typedef int cgsize_t;
typedef enum { ZoneTypeNull = 0, ZoneTypeUserDefined, Structured, Unstructured } ZoneType_t;
typedef enum { DataTypeNull = 0, DataTypeUserDefined, Integer, RealSingle, RealDouble, Character, LongInteger } DataType_t;
typedef enum {
  ElementTypeNull = 0, ElementTypeUserDefined, NODE, BAR_2, BAR_3, TRI_3, TRI_6, QUAD_4, QUAD_8, QUAD_9, TETRA_4,
  TETRA_10, PYRA_5, PYRA_14, PENTA_6, PENTA_15, PENTA_18, HEXA_8, HEXA_20, HEXA_27, MIXED
} ElementType_t;
#ifdef __cplusplus
extern "C" {
#endif
#define CG_MODE_READ 0
#define CG_OK 0
#define CG_ERROR 1
extern const char* DataTypeName[];
const char* cg_get_error();
const char* cg_ZoneTypeName(ZoneType_t t);
const char* cg_ElementTypeName(ElementType_t t);
int cg_open(const char* name, int mode, int* fn);
int cg_close(int fn);
int cg_version(int fn, float* version);
int cg_zone_read(int fn, int b, int z, char* name, cgsize_t* size);
int cg_zone_type(int fn, int b, int z, ZoneType_t* t);
int cg_ncoords(int fn, int b, int z, int* n);
int cg_coord_info(int fn, int b, int z, int c, DataType_t* t, char* name);
int cg_coord_read(int fn, int b, int z, const char* name, DataType_t t, const cgsize_t* rmin, const cgsize_t* rmax,
                  void* data);
int cg_nsections(int fn, int b, int z, int* n);
int cg_section_read(int fn, int b, int z, int s, char* name, ElementType_t* t, cgsize_t* start, cgsize_t* end,
                    int* nbndry, int* parent_flag);
int cg_ElementDataSize(int fn, int b, int z, int s, cgsize_t* size);
int cg_elements_read(int fn, int b, int z, int s, cgsize_t* elements, cgsize_t* parent);
int cg_npe(ElementType_t t, int* npe);
#ifdef __cplusplus
}
#endif
