/*
 * lagrbf_petsc_gpu.h -- in-process GPU plug-ins for LagRBF's own C code (one MPI rank), on top of
 * the C-ABI of liblagrbf.so (include/lagrbf.h).
 *
 * Every function has the exact signature of the reference plug-in point it replaces:
 *   LagRBFGPU_RBFInterpolation       RBFInterpolation            (include/interpolation.h:34)
 *   LagRBFGPU_SwarmInterpSetWeights  SwarmInterpSetWeights       (include/swarm/swarm_interp.h:35)
 *   LagRBFGPU_PartitionSetUp         PartitionOfUnity->psetup    (include/partition_of_unity.h:51)
 *   LagRBFGPU_PartitionSolve         PartitionOfUnity->psolve    (include/partition_of_unity.h:53)
 *   LagRBFGPU_PartitionDestroy       PartitionOfUnity->pdestroy  (include/partition_of_unity.h:52)
 *   LagRBFGPU_AdvectionStep          AdvectionCtx->advection     (include/advection/advection_ctx.h:55)
 * LagRBFGPU_Attach(ctx) creates the GPU context from the LagRBFCtx (mesh, kernel, solve method,
 * fields, advection scheme and step) and installs the four function-pointer plug-ins, so the
 * reference's time loop runs unchanged: LagRBF_PartitionsSetUp calls the no-op psetup/psolve (the
 * GPU sets up and solves the same lazily touched patches, batched, inside the interpolation), and
 * the advection pointer advances the swarm on the GPU.  The two compile-time dispatch sites
 * (RBFInterpolation, interpolation.c:217-262; SwarmInterpSetWeights, swarm_interp.c:382-396) call
 * the GPU functions from a LAGRBF_GPU branch, or, compiled with -DLAGRBF_GPU_REPLACE, this unit
 * defines them under the reference names for builds that leave out those two definitions.
 * Headers are the reference's, unchanged; PetscErrorCode values are the C-ABI's (PETSc numbering).
 */
#ifndef LAGRBF_PETSC_GPU_H
#define LAGRBF_PETSC_GPU_H

#include <petsc.h>
#include "lagrangian_rbf.h"
#include "interpolation.h"
#include "partition_of_unity.h"
#include "advection/advection_ctx.h"
#include "swarm/swarm_interp.h"

PetscErrorCode LagRBFGPU_Attach(LagRBFCtx ctx);
PetscErrorCode LagRBFGPU_Detach(LagRBFCtx ctx);
PetscErrorCode LagRBFGPU_RBFInterpolation(LagRBFCtx ctx, DM swi, DM swd, const char *fieldname);
PetscErrorCode LagRBFGPU_SwarmInterpSetWeights(LagRBFCtx ctx, DM sw);
PetscErrorCode LagRBFGPU_PartitionSetUp(LagRBFCtx ctx, Partition p, PetscReal *data);
PetscErrorCode LagRBFGPU_PartitionSolve(LagRBFCtx ctx, Partition p, PetscInt nfields, PetscReal *data);
PetscErrorCode LagRBFGPU_PartitionDestroy(Partition p);
PetscErrorCode LagRBFGPU_AdvectionStep(LagRBFCtx ctx, DM swi, DM swd);

#endif
