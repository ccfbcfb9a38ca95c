// Single-rank stand-in for the PETSc system interface the reference calls (TEST INFRASTRUCTURE
// ONLY).  Options come from the command line given to PetscInitialize ("-name value" pairs);
// log stages are counted and otherwise ignored.  Implemented in oracle/refpin/refpin_runtime.cpp.
#pragma once
#include <cstddef>
#include <cstdio>
#include "mpi.h"

typedef int PetscErrorCode;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef double PetscScalar;
typedef double PetscReal;
typedef int PetscLogStage;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
struct refpin_viewer;
typedef refpin_viewer* PetscViewer;
struct refpin_options;
typedef refpin_options* PetscOptions;

#define PETSC_DEFAULT -2
#define PETSC_DECIDE -1
#define PETSC_NULL 0
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)
#define CHKERRQ(e) do { if (e) return (e); } while (0)

PetscErrorCode PetscInitialize(int* argc, char*** argv, const char* file, const char* help);
PetscErrorCode PetscFinalize();
PetscErrorCode PetscPrintf(MPI_Comm comm, const char* fmt, ...);
PetscErrorCode PetscOptionsGetString(PetscOptions opts, const char* pre, const char* name, char* value, size_t len,
                                     PetscBool* set);
PetscErrorCode PetscOptionsGetBool(PetscOptions opts, const char* pre, const char* name, PetscBool* value,
                                   PetscBool* set);
PetscErrorCode PetscLogStageRegister(const char* name, PetscLogStage* stage);
PetscErrorCode PetscLogStagePush(PetscLogStage stage);
PetscErrorCode PetscLogStagePop();
