/* ORACLE BUILD SUPPORT (test infrastructure only): the PETSc names the reference's headers use, for one
 * process. Vec is a plain array with an optional ghost tail (ref_stubs.cpp); matrices, solvers and viewers are
 * declared only. */
#ifndef REF_STUB_PETSC_H
#define REF_STUB_PETSC_H

#include "stub_core.h"

#define PETSC_VERSION_MAJOR 3
#define PETSC_VERSION_MINOR 16
#define PETSC_VERSION_SUBMINOR 3
#define PETSC_VERSION_RELEASE 1
#define PETSC_VERSION_LT(a, b, c) \
  (PETSC_VERSION_MAJOR < (a) || (PETSC_VERSION_MAJOR == (a) && (PETSC_VERSION_MINOR < (b) || (PETSC_VERSION_MINOR == (b) && PETSC_VERSION_SUBMINOR < (c)))))
#define PETSC_VERSION_LE(a, b, c) (PETSC_VERSION_LT(a, b, c) || (PETSC_VERSION_MAJOR == (a) && PETSC_VERSION_MINOR == (b) && PETSC_VERSION_SUBMINOR == (c)))
#define PETSC_VERSION_GE(a, b, c) (!PETSC_VERSION_LT(a, b, c))
#define PETSC_VERSION_GT(a, b, c) (!PETSC_VERSION_LE(a, b, c))

#ifdef __cplusplus
extern "C" {
#endif

typedef int PetscErrorCode;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef double PetscScalar;
typedef double PetscReal;
typedef double PetscLogDouble;
typedef int PetscLogEvent;
typedef int PetscLogStage;
typedef int PetscClassId;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES, MAX_VALUES, MIN_VALUES } InsertMode;
typedef enum { SCATTER_FORWARD = 0, SCATTER_REVERSE = 1, SCATTER_FORWARD_LOCAL = 2, SCATTER_REVERSE_LOCAL = 3 } ScatterMode;
typedef enum { NORM_1 = 0, NORM_2 = 1, NORM_FROBENIUS = 2, NORM_INFINITY = 3, NORM_1_AND_2 = 4 } NormType;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { PETSC_COPY_VALUES, PETSC_OWN_POINTER, PETSC_USE_POINTER } PetscCopyMode;
typedef enum { FILE_MODE_READ, FILE_MODE_WRITE, FILE_MODE_APPEND } PetscFileMode;
typedef enum { MAT_INITIAL_MATRIX, MAT_REUSE_MATRIX } MatReuse;
typedef enum { DIFFERENT_NONZERO_PATTERN, SUBSET_NONZERO_PATTERN, SAME_NONZERO_PATTERN } MatStructure;
typedef enum { MAT_NEW_NONZERO_ALLOCATION_ERR = 19, MAT_NO_OFF_PROC_ENTRIES = 0, MAT_SYMMETRIC = 1 } MatOption;
typedef enum { KSP_NORM_DEFAULT = -1, KSP_NORM_NONE = 0, KSP_NORM_PRECONDITIONED = 1, KSP_NORM_UNPRECONDITIONED = 2 } KSPNormType;
typedef int KSPConvergedReason;
typedef const char *KSPType;
typedef const char *PCType;
typedef const char *MatType;
typedef const char *VecType;

typedef struct ref_vec_s *Vec;
typedef struct ref_opaque_s *Mat;
typedef struct ref_opaque_s *KSP;
typedef struct ref_opaque_s *PC;
typedef struct ref_opaque_s *IS;
typedef struct ref_opaque_s *ISLocalToGlobalMapping;
typedef struct ref_opaque_s *VecScatter;
typedef struct ref_opaque_s *PetscViewer;
typedef struct ref_opaque_s *MatNullSpace;
typedef struct ref_opaque_s *AO;
typedef struct ref_opaque_s *PetscRandom;
typedef struct ref_opaque_s *SNES;
typedef struct ref_opaque_s *TS;

#define PETSC_COMM_WORLD MPI_COMM_WORLD
#define PETSC_COMM_SELF MPI_COMM_SELF
#define PETSC_DECIDE (-1)
#define PETSC_DETERMINE (-1)
#define PETSC_DEFAULT (-2)
#define PETSC_NULL 0
#define PETSC_MAX_REAL 1.7976931348623157e308
#define PETSC_MIN_REAL (-1.7976931348623157e308)
#define PETSC_INFINITY PETSC_MAX_REAL
#define PETSC_MACHINE_EPSILON 2.2204460492503131e-16
#define PETSC_SUCCESS 0
#define PETSC_ERR_ARG_WRONG 62
#define PETSC_ERR_ARG_OUTOFRANGE 63
#define PETSC_ERR_SUP 56
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)
#define PETSC_VIEWER_STDOUT_SELF ((PetscViewer)0)
#define MPIU_REAL MPI_DOUBLE
#define MPIU_SCALAR MPI_DOUBLE
#define MPIU_INT MPI_INT
#define MPIU_BOOL MPI_INT
#define KSPBCGS "bcgs"
#define KSPCG "cg"
#define KSPGMRES "gmres"
#define PCHYPRE "hypre"
#define PCSOR "sor"
#define PCJACOBI "jacobi"
#define PCNONE "none"
#define PCLU "lu"
#define MATAIJ "aij"
#define MATMPIAIJ "mpiaij"
#define VECMPI "mpi"
#define PETSC_VIEWER_ASCII_INFO 0

#define CHKERRABORT(comm, ierr) do { if (ierr) { fprintf(stderr, "reference stub: error %d at %s:%d\n", (int)(ierr), __FILE__, __LINE__); abort(); } } while (0)
#define CHKERRQ(ierr) do { if (ierr) return ierr; } while (0)
#define CHKERRV(ierr) do { if (ierr) return; } while (0)
#define CHKERRMPI(ierr) CHKERRQ(ierr)
#define SETERRQ(comm, code, ...) return (code)
#define PetscFunctionBegin
#define PetscFunctionBeginUser
#define PetscFunctionReturn(x) return (x)

PetscErrorCode PetscLogFlops(PetscLogDouble);
PetscErrorCode PetscLogEventBegin(PetscLogEvent, ...);
PetscErrorCode PetscLogEventEnd(PetscLogEvent, ...);
PetscErrorCode PetscLogEventRegister(const char *, PetscClassId, PetscLogEvent *);
PetscErrorCode PetscPrintf(MPI_Comm, const char *, ...);
PetscErrorCode PetscFPrintf(MPI_Comm, FILE *, const char *, ...);
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm, const char *, ...);
PetscErrorCode PetscSynchronizedFPrintf(MPI_Comm, FILE *, const char *, ...);
PetscErrorCode PetscSynchronizedFlush(MPI_Comm, FILE *);
PetscErrorCode PetscFOpen(MPI_Comm, const char *, const char *, FILE **);
PetscErrorCode PetscFClose(MPI_Comm, FILE *);
PetscErrorCode PetscInitialize(int *, char ***, const char *, const char *);
PetscErrorCode PetscFinalize(void);
PetscErrorCode PetscTime(PetscLogDouble *);
PetscErrorCode PetscMalloc(size_t, void *);
PetscErrorCode PetscFree(void *);
PetscErrorCode PetscOptionsSetValue(void *, const char *, const char *);
PetscErrorCode PetscOptionsGetInt(void *, const char *, const char *, PetscInt *, PetscBool *);

/* Vec (functional on one process) */
PetscErrorCode VecCreate(MPI_Comm, Vec *);
PetscErrorCode VecCreateSeq(MPI_Comm, PetscInt, Vec *);
PetscErrorCode VecCreateMPI(MPI_Comm, PetscInt, PetscInt, Vec *);
PetscErrorCode VecCreateGhost(MPI_Comm, PetscInt, PetscInt, PetscInt, const PetscInt[], Vec *);
PetscErrorCode VecCreateGhostBlock(MPI_Comm, PetscInt, PetscInt, PetscInt, PetscInt, const PetscInt[], Vec *);
PetscErrorCode VecDuplicate(Vec, Vec *);
PetscErrorCode VecDestroy(Vec *);
PetscErrorCode VecCopy(Vec, Vec);
PetscErrorCode VecSet(Vec, PetscScalar);
PetscErrorCode VecScale(Vec, PetscScalar);
PetscErrorCode VecShift(Vec, PetscScalar);
PetscErrorCode VecAXPY(Vec, PetscScalar, Vec);
PetscErrorCode VecAXPBY(Vec, PetscScalar, PetscScalar, Vec);
PetscErrorCode VecAYPX(Vec, PetscScalar, Vec);
PetscErrorCode VecWAXPY(Vec, PetscScalar, Vec, Vec);
PetscErrorCode VecPointwiseMult(Vec, Vec, Vec);
PetscErrorCode VecPointwiseDivide(Vec, Vec, Vec);
PetscErrorCode VecPointwiseMax(Vec, Vec, Vec);
PetscErrorCode VecPointwiseMin(Vec, Vec, Vec);
PetscErrorCode VecReciprocal(Vec);
PetscErrorCode VecAbs(Vec);
PetscErrorCode VecSqrtAbs(Vec);
PetscErrorCode VecNorm(Vec, NormType, PetscReal *);
PetscErrorCode VecMax(Vec, PetscInt *, PetscReal *);
PetscErrorCode VecMin(Vec, PetscInt *, PetscReal *);
PetscErrorCode VecSum(Vec, PetscScalar *);
PetscErrorCode VecDot(Vec, Vec, PetscScalar *);
PetscErrorCode VecGetSize(Vec, PetscInt *);
PetscErrorCode VecGetLocalSize(Vec, PetscInt *);
PetscErrorCode VecGetBlockSize(Vec, PetscInt *);
PetscErrorCode VecSetBlockSize(Vec, PetscInt);
PetscErrorCode VecGetOwnershipRange(Vec, PetscInt *, PetscInt *);
PetscErrorCode VecGetArray(Vec, PetscScalar **);
PetscErrorCode VecRestoreArray(Vec, PetscScalar **);
PetscErrorCode VecGetArrayRead(Vec, const PetscScalar **);
PetscErrorCode VecRestoreArrayRead(Vec, const PetscScalar **);
PetscErrorCode VecGhostGetLocalForm(Vec, Vec *);
PetscErrorCode VecGhostRestoreLocalForm(Vec, Vec *);
PetscErrorCode VecGhostUpdateBegin(Vec, InsertMode, ScatterMode);
PetscErrorCode VecGhostUpdateEnd(Vec, InsertMode, ScatterMode);
PetscErrorCode VecSetValue(Vec, PetscInt, PetscScalar, InsertMode);
PetscErrorCode VecSetValues(Vec, PetscInt, const PetscInt[], const PetscScalar[], InsertMode);
PetscErrorCode VecSetValuesLocal(Vec, PetscInt, const PetscInt[], const PetscScalar[], InsertMode);
PetscErrorCode VecAssemblyBegin(Vec);
PetscErrorCode VecAssemblyEnd(Vec);
PetscErrorCode VecSetFromOptions(Vec);
PetscErrorCode VecSetSizes(Vec, PetscInt, PetscInt);
PetscErrorCode VecSetType(Vec, VecType);
PetscErrorCode VecView(Vec, PetscViewer);
PetscErrorCode VecLoad(Vec, PetscViewer);
PetscErrorCode VecSetLocalToGlobalMapping(Vec, ISLocalToGlobalMapping);
PetscErrorCode VecGetLocalToGlobalMapping(Vec, ISLocalToGlobalMapping *);
PetscErrorCode VecScatterCreate(Vec, IS, Vec, IS, VecScatter *);
PetscErrorCode VecScatterBegin(VecScatter, Vec, Vec, InsertMode, ScatterMode);
PetscErrorCode VecScatterEnd(VecScatter, Vec, Vec, InsertMode, ScatterMode);
PetscErrorCode VecScatterDestroy(VecScatter *);
PetscErrorCode VecStrideGather(Vec, PetscInt, Vec, InsertMode);
PetscErrorCode VecStrideScatter(Vec, PetscInt, Vec, InsertMode);
PetscErrorCode VecMDot(Vec, PetscInt, const Vec[], PetscScalar[]);
PetscErrorCode VecGetArrayWrite(Vec, PetscScalar **);
PetscErrorCode VecRestoreArrayWrite(Vec, PetscScalar **);
PetscErrorCode VecGetType(Vec, VecType *);

PetscErrorCode ISCreateGeneral(MPI_Comm, PetscInt, const PetscInt[], PetscCopyMode, IS *);
PetscErrorCode ISCreateBlock(MPI_Comm, PetscInt, PetscInt, const PetscInt[], PetscCopyMode, IS *);
PetscErrorCode ISDestroy(IS *);
PetscErrorCode ISCreateStride(MPI_Comm, PetscInt, PetscInt, PetscInt, IS *);
PetscErrorCode ISLocalToGlobalMappingGetIndices(ISLocalToGlobalMapping, const PetscInt **);
PetscErrorCode ISLocalToGlobalMappingRestoreIndices(ISLocalToGlobalMapping, const PetscInt **);
PetscErrorCode ISLocalToGlobalMappingGetSize(ISLocalToGlobalMapping, PetscInt *);
PetscErrorCode ISLocalToGlobalMappingCreate(MPI_Comm, PetscInt, PetscInt, const PetscInt[], PetscCopyMode, ISLocalToGlobalMapping *);
PetscErrorCode ISLocalToGlobalMappingDestroy(ISLocalToGlobalMapping *);
PetscErrorCode ISLocalToGlobalMappingApply(ISLocalToGlobalMapping, PetscInt, const PetscInt[], PetscInt[]);

PetscErrorCode PetscViewerBinaryOpen(MPI_Comm, const char[], PetscFileMode, PetscViewer *);
PetscErrorCode PetscViewerDestroy(PetscViewer *);
PetscErrorCode PetscViewerASCIIOpen(MPI_Comm, const char[], PetscViewer *);
PetscErrorCode PetscViewerPushFormat(PetscViewer, int);
PetscErrorCode PetscViewerPopFormat(PetscViewer);
PetscErrorCode PetscBinaryWrite(int, const void *, PetscInt, int);
PetscErrorCode PetscBinaryRead(int, void *, PetscInt, PetscInt *, int);

PetscErrorCode MatCreate(MPI_Comm, Mat *);
PetscErrorCode MatDestroy(Mat *);
PetscErrorCode MatSetType(Mat, MatType);
PetscErrorCode MatSetSizes(Mat, PetscInt, PetscInt, PetscInt, PetscInt);
PetscErrorCode MatSetFromOptions(Mat);
PetscErrorCode MatSetOption(Mat, MatOption, PetscBool);
PetscErrorCode MatSetValue(Mat, PetscInt, PetscInt, PetscScalar, InsertMode);
PetscErrorCode MatSetValues(Mat, PetscInt, const PetscInt[], PetscInt, const PetscInt[], const PetscScalar[], InsertMode);
PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType);
PetscErrorCode MatAssemblyEnd(Mat, MatAssemblyType);
PetscErrorCode MatMult(Mat, Vec, Vec);
PetscErrorCode MatMultAdd(Mat, Vec, Vec, Vec);
PetscErrorCode MatGetDiagonal(Mat, Vec);
PetscErrorCode MatDiagonalSet(Mat, Vec, InsertMode);
PetscErrorCode MatZeroEntries(Mat);
PetscErrorCode MatMPIAIJSetPreallocation(Mat, PetscInt, const PetscInt[], PetscInt, const PetscInt[]);
PetscErrorCode MatSeqAIJSetPreallocation(Mat, PetscInt, const PetscInt[]);
PetscErrorCode MatNullSpaceCreate(MPI_Comm, PetscBool, PetscInt, const Vec[], MatNullSpace *);
PetscErrorCode MatNullSpaceDestroy(MatNullSpace *);
PetscErrorCode MatNullSpaceRemove(MatNullSpace, Vec);
PetscErrorCode MatSetNullSpace(Mat, MatNullSpace);
PetscErrorCode MatShift(Mat, PetscScalar);
PetscErrorCode MatScale(Mat, PetscScalar);
PetscErrorCode MatGetOwnershipRange(Mat, PetscInt *, PetscInt *);
PetscErrorCode MatView(Mat, PetscViewer);
PetscErrorCode MatAXPY(Mat, PetscScalar, Mat, MatStructure);
PetscErrorCode MatDuplicate(Mat, int, Mat *);
PetscErrorCode MatGetSize(Mat, PetscInt *, PetscInt *);
PetscErrorCode MatGetLocalSize(Mat, PetscInt *, PetscInt *);
PetscErrorCode MatGetRow(Mat, PetscInt, PetscInt *, const PetscInt *[], const PetscScalar *[]);
PetscErrorCode MatRestoreRow(Mat, PetscInt, PetscInt *, const PetscInt *[], const PetscScalar *[]);
PetscErrorCode MatCopy(Mat, Mat, MatStructure);
PetscErrorCode MatTranspose(Mat, MatReuse, Mat *);
PetscErrorCode MatMatMult(Mat, Mat, MatReuse, PetscReal, Mat *);

PetscErrorCode KSPCreate(MPI_Comm, KSP *);
PetscErrorCode KSPDestroy(KSP *);
PetscErrorCode KSPSetType(KSP, KSPType);
PetscErrorCode KSPSetOperators(KSP, Mat, Mat);
PetscErrorCode KSPSolve(KSP, Vec, Vec);
PetscErrorCode KSPGetPC(KSP, PC *);
PetscErrorCode KSPSetTolerances(KSP, PetscReal, PetscReal, PetscReal, PetscInt);
PetscErrorCode KSPSetFromOptions(KSP);
PetscErrorCode KSPSetUp(KSP);
PetscErrorCode KSPSetInitialGuessNonzero(KSP, PetscBool);
PetscErrorCode KSPGetConvergedReason(KSP, KSPConvergedReason *);
PetscErrorCode KSPGetIterationNumber(KSP, PetscInt *);
PetscErrorCode KSPSetNormType(KSP, KSPNormType);
PetscErrorCode KSPGetType(KSP, KSPType *);
PetscErrorCode KSPSetNullSpace(KSP, MatNullSpace);
PetscErrorCode KSPGetResidualNorm(KSP, PetscReal *);
PetscErrorCode PCSetType(PC, PCType);
PetscErrorCode PCSetFromOptions(PC);
PetscErrorCode PCGetType(PC, PCType *);
PetscErrorCode PCFactorSetShiftType(PC, int);

#ifdef __cplusplus
}
#endif

#endif
