/*
 * petsc.h -- minimal stand-in for the PETSc API surface used by LagRBF's hot-loop translation
 * units, so that those units compile unmodified, in place, into a test-only library that checks
 * the oracle (TEST INFRASTRUCTURE ONLY: never linked into liblagrbf.so).  The GPU plug-ins of
 * lagrbf_gb300/adapters/petsc are compile-checked against the reference headers with it too.
 *
 * Types follow the reference's PETSc configuration (32-bit indices, double precision):
 * PetscInt = int32_t, PetscReal = PetscScalar = double.  DM / Mat / Vec are handles to the small
 * array-backed objects defined in refpin.c; only the calls the compiled units make exist.
 */
#ifndef LAGRBF_REFPIN_PETSC_SHIM_H
#define LAGRBF_REFPIN_PETSC_SHIM_H

#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef int32_t PetscInt;
typedef int64_t PetscInt64;
typedef int PetscMPIInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef int PetscErrorCode;
typedef int PetscLogEvent;
typedef int PetscDataType;
typedef int MPI_Comm;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES } InsertMode;

typedef struct rp_dm *DM;
typedef struct rp_mat *Mat;
typedef struct rp_vec *Vec;
typedef struct rp_ksp *KSP;
typedef struct rp_celldm *DMSwarmCellDM;

#define PETSC_SUCCESS 0
#define PETSC_ERR_SUP 56
#define PETSC_ERR_ARG_WRONG 62
#define PETSC_ERR_ARG_OUTOFRANGE 63
#define PETSC_ERR_ARG_WRONGSTATE 73
#define PETSC_ERR_PLIB 77
#define PETSC_COMM_SELF 0
#define PETSC_COMM_WORLD 1
#define PETSC_MAX_PATH_LEN 4096
#define PETSC_FUNCTION_NAME __func__
#define PETSC_MAX_REAL 1.7976931348623157e+308
#define PetscInt_FMT "d"

#define PetscFunctionBeginUser do { } while (0)
#define PetscFunctionReturn(x) return (x)
#define PetscCall(x)                                                                               \
  do {                                                                                             \
    PetscErrorCode rp_e_ = (x);                                                                    \
    if (rp_e_) return rp_e_;                                                                       \
  } while (0)
#define SETERRQ(comm, code, ...) return rp_seterr((code), __VA_ARGS__)

#define PetscLogEventBegin(e, a, b, c, d) 0
#define PetscLogEventEnd(e, a, b, c, d) 0
#define PetscCalloc1(n, p) rp_calloc((size_t)(n) * sizeof(**(p)), (void **)(p))
#define PetscFree(p) (free(p), (p) = NULL, 0)
#define PetscArrayzero(p, n) (memset((p), 0, (size_t)(n) * sizeof(*(p))), 0)
#define PetscSqrtReal(x) sqrt(x)
#define PetscExpReal(x) exp(x)
#define PetscPowReal(x, y) pow((x), (y))
#define PetscAbsReal(x) fabs(x)

PetscErrorCode rp_seterr(PetscErrorCode code, const char *fmt, ...);
PetscErrorCode rp_calloc(size_t bytes, void **p);
PetscErrorCode PetscPrintf(MPI_Comm comm, const char *fmt, ...);

PetscErrorCode DMGetDimension(DM dm, PetscInt *dim);
PetscErrorCode DMGetCoordinateDM(DM dm, DM *cdm);
PetscErrorCode DMGetCoordinates(DM dm, Vec *coords);
PetscErrorCode DMDAGetElements(DM dm, PetscInt *nel, PetscInt *nen, const PetscInt **e);
PetscErrorCode DMDARestoreElements(DM dm, PetscInt *nel, PetscInt *nen, const PetscInt **e);
PetscErrorCode VecGetArray(Vec v, PetscScalar **a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a);
PetscErrorCode MatDenseGetArray(Mat m, PetscScalar **a);
PetscErrorCode MatDenseRestoreArray(Mat m, PetscScalar **a);
PetscErrorCode DMSwarmGetLocalSize(DM sw, PetscInt *n);
PetscErrorCode DMSwarmGetCellDMActive(DM sw, DMSwarmCellDM *celldm);
PetscErrorCode DMSwarmCellDMGetCoordinateFields(DMSwarmCellDM celldm, PetscInt *nf, const char ***names);
PetscErrorCode DMSwarmCellDMGetCellID(DMSwarmCellDM celldm, const char **name);
PetscErrorCode DMSwarmGetField(DM sw, const char *name, PetscInt *bs, PetscDataType *type, void **data);
PetscErrorCode DMSwarmRestoreField(DM sw, const char *name, PetscInt *bs, PetscDataType *type, void **data);
/* declared for the compile check of the GPU plug-ins (lagrbf_gb300/adapters/petsc); not defined */
#define DMSwarmField_pid "DMSwarm_pid"
PetscErrorCode DMSwarmRemovePointAtIndex(DM sw, PetscInt idx);

#endif
