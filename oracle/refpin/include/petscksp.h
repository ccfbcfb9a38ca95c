// Single-rank stand-in for the PETSc Vec / Mat / KSP interface the reference calls (TEST
// INFRASTRUCTURE ONLY).
//
// Vec: a contiguous double array (owned, or borrowed from the caller as VecCreateMPIWithArray
// does).  Mat: an AIJ-like matrix whose pattern is the union of every (row, column) ever set --
// explicit zeros included, as AIJ keeps them -- with columns sorted within each row;
// MatZeroEntries keeps the pattern.  KSP: GMRES or CG with ILU(0) (PETSc's default on one rank),
// Jacobi or no preconditioner, solved by the oracle's restatement of PETSc's published
// algorithms (oracle/oracle_krylov.cpp), so the Krylov arithmetic on this side is the
// oracle's and everything around it is the reference's own code.  Implemented in
// oracle/refpin/refpin_runtime.cpp.
#pragma once
#include "petscsys.h"

struct refpin_vec;
struct refpin_mat;
struct refpin_ksp;
typedef refpin_vec* Vec;
typedef refpin_mat* Mat;
typedef refpin_ksp* KSP;
typedef refpin_ksp* PC;
typedef const char* MatType;
typedef const char* KSPType;
typedef int KSPConvergedReason;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_INFINITY = 3 } NormType;
typedef enum { INSERT_VALUES = 1, ADD_VALUES = 2 } InsertMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { MAT_SYMMETRIC = 1, MAT_STRUCTURALLY_SYMMETRIC = 2 } MatOption;

#define MATAIJ "aij"
#define KSPGMRES "gmres"
#define KSPCG "cg"

PetscErrorCode VecCreateMPI(MPI_Comm comm, PetscInt n, PetscInt N, Vec* v);
PetscErrorCode VecCreateMPIWithArray(MPI_Comm comm, PetscInt bs, PetscInt n, PetscInt N, const PetscScalar* array,
                                     Vec* v);
PetscErrorCode VecDuplicate(Vec v, Vec* out);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar a, InsertMode mode);
PetscErrorCode VecAssemblyBegin(Vec v);
PetscErrorCode VecAssemblyEnd(Vec v);
PetscErrorCode VecNorm(Vec v, NormType type, PetscReal* out);
PetscErrorCode VecGetArray(Vec v, PetscScalar** a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar** a);
PetscErrorCode VecView(Vec v, PetscViewer viewer);
PetscErrorCode VecDestroy(Vec* v);

PetscErrorCode MatCreate(MPI_Comm comm, Mat* m);
PetscErrorCode MatSetSizes(Mat m, PetscInt n, PetscInt nc, PetscInt N, PetscInt Nc);
PetscErrorCode MatSetType(Mat m, MatType type);
PetscErrorCode MatMPIAIJSetPreallocation(Mat m, PetscInt dnz, const PetscInt* dnnz, PetscInt onz,
                                         const PetscInt* onnz);
PetscErrorCode MatSetValue(Mat m, PetscInt i, PetscInt j, PetscScalar v, InsertMode mode);
PetscErrorCode MatSetValues(Mat m, PetscInt nr, const PetscInt* rows, PetscInt nc, const PetscInt* cols,
                            const PetscScalar* v, InsertMode mode);
PetscErrorCode MatAssemblyBegin(Mat m, MatAssemblyType type);
PetscErrorCode MatAssemblyEnd(Mat m, MatAssemblyType type);
PetscErrorCode MatZeroEntries(Mat m);
PetscErrorCode MatSetOption(Mat m, MatOption op, PetscBool flag);
PetscErrorCode MatGetOwnershipRange(Mat m, PetscInt* lo, PetscInt* hi);
PetscErrorCode MatView(Mat m, PetscViewer viewer);
PetscErrorCode MatDestroy(Mat* m);

PetscErrorCode KSPCreate(MPI_Comm comm, KSP* ksp);
PetscErrorCode KSPSetOperators(KSP ksp, Mat A, Mat P);
PetscErrorCode KSPSetType(KSP ksp, KSPType type);
PetscErrorCode KSPSetInitialGuessNonzero(KSP ksp, PetscBool flag);
PetscErrorCode KSPSetTolerances(KSP ksp, PetscReal rtol, PetscReal abstol, PetscReal dtol, PetscInt maxits);
PetscErrorCode KSPSetFromOptions(KSP ksp);
PetscErrorCode KSPSetUp(KSP ksp);
PetscErrorCode KSPSolve(KSP ksp, Vec b, Vec x);
PetscErrorCode KSPGetConvergedReason(KSP ksp, KSPConvergedReason* reason);
PetscErrorCode KSPGetIterationNumber(KSP ksp, PetscInt* its);
PetscErrorCode KSPGetResidualNorm(KSP ksp, PetscReal* rnorm);
PetscErrorCode KSPGetPC(KSP ksp, PC* pc);
PetscErrorCode KSPView(KSP ksp, PetscViewer viewer);
PetscErrorCode KSPDestroy(KSP* ksp);
