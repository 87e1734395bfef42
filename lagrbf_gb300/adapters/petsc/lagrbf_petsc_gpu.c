/*
 * lagrbf_petsc_gpu.c -- in-process GPU plug-ins for LagRBF's own C code (see lagrbf_petsc_gpu.h).
 *
 * Built with the reference's headers and PETSc (only when PETSC_DIR is set; one MPI rank), linked
 * with liblagrbf.so.  The DMSwarm fields are read and written in place through DMSwarmGetField /
 * DMSwarmRestoreField; the C-ABI copies the inputs and writes the outputs by pid, so the swarm's
 * order, sizes and pids stay PETSc's.
 */
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include "lagrbf_petsc_gpu.h"
#include "lagrbf.h" /* include/ of liblagrbf */

/* GPU context of each attached LagRBFCtx. */
#define LAGRBF_GPU_MAXCTX 64
static struct { LagRBFCtx ctx; void *gpu; } g_attached[LAGRBF_GPU_MAXCTX];

static void *gpu_of(LagRBFCtx ctx)
{
  int i;
  for (i = 0; i < LAGRBF_GPU_MAXCTX; i++)
    if (g_attached[i].ctx == ctx) return g_attached[i].gpu;
  return NULL;
}

static int set_opt(const char *key, const char *fmt, ...)
{
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  return lagrbf_options_set_value(key, buf);
}

static int set_array(const char *key, const PetscReal *v, PetscInt n)
{
  char buf[512];
  int len = 0, i;
  for (i = 0; i < n; i++) len += snprintf(buf + len, sizeof(buf) - (size_t)len, i ? ",%.17g" : "%.17g", v[i]);
  return lagrbf_options_set_value(key, buf);
}

PetscErrorCode LagRBFGPU_Attach(LagRBFCtx ctx)
{
  PartitionOfUnity pu = ctx->pu;
  PetscInt i, n[3] = {0, 0, 0};
  void *gpu;
  char nb[64];
  int slot = -1;
  if (gpu_of(ctx)) return 0;
  for (i = 0; i < LAGRBF_GPU_MAXCTX && slot < 0; i++)
    if (!g_attached[i].ctx) slot = (int)i;
  if (slot < 0) return LAGRBF_ERR_MEM;
  for (i = 0; i < pu->dim; i++) n[i] = pu->n[i];
  snprintf(nb, sizeof(nb), pu->dim == 3 ? "%d,%d,%d" : "%d,%d", (int)n[0], (int)n[1], (int)n[2]);
  /* LagRBFSetFromOptions / PUSetFromOptions keys, from the context itself */
  if (set_opt("pu_mesh_dim", "%d", (int)pu->dim) || lagrbf_options_set_value("pu_mesh_n", nb) ||
      set_array("pu_mesh_O", pu->O, pu->dim) || set_array("pu_mesh_L", pu->L, pu->dim) ||
      set_opt("pu_mesh_overlap", "%.17g", pu->overlap) || set_opt("pu_mesh_shape_factor", "%.17g", pu->shape_fac) ||
      set_opt("kernel_type", "%d", (int)ctx->kernel_type) || set_opt("solve_method", "%d", (int)ctx->solve_method) ||
      set_opt("n_interpolation_fields", "%d", (int)ctx->n_ifields) || set_opt("cfl_fac", "%.17g", ctx->cfl_fac) ||
      set_opt("rmin", "%.17g", ctx->rmin) || set_opt("rmax", "%.17g", ctx->rmax) ||
      set_opt("advection", "%s", ctx->advection ? "true" : "false"))
    return LAGRBF_ERR_MEM;
  if (ctx->advection && ctx->adv_ctx &&
      (set_opt("advection_scheme", "%d", (int)ctx->adv_ctx->scheme) || set_opt("dt", "%.17g", ctx->adv_ctx->dt)))
    return LAGRBF_ERR_MEM;
  gpu = lagrbf_create();
  if (!gpu) return LAGRBF_ERR_GPU;
  g_attached[slot].ctx = ctx;
  g_attached[slot].gpu = gpu;
  /* the function-pointer plug-ins */
  pu->psetup = LagRBFGPU_PartitionSetUp;
  pu->psolve = LagRBFGPU_PartitionSolve;
  pu->pdestroy = LagRBFGPU_PartitionDestroy;
  pu->psetup_set = PETSC_TRUE;
  if (ctx->adv_ctx) ctx->adv_ctx->advection = LagRBFGPU_AdvectionStep;
  return 0;
}

PetscErrorCode LagRBFGPU_Detach(LagRBFCtx ctx)
{
  int i;
  for (i = 0; i < LAGRBF_GPU_MAXCTX; i++)
    if (g_attached[i].ctx == ctx) {
      lagrbf_destroy(g_attached[i].gpu);
      g_attached[i].ctx = NULL;
      g_attached[i].gpu = NULL;
    }
  return 0;
}

/* Patch set-up and solve are batched on the GPU inside the interpolation (lagrbf_interpolation
   sets up and solves the patches touched by the particles, as LagRBF_PartitionsSetUp does): the
   per-partition plug-ins have nothing left to do. */
PetscErrorCode LagRBFGPU_PartitionSetUp(LagRBFCtx ctx, Partition p, PetscReal *data) { return 0; }
PetscErrorCode LagRBFGPU_PartitionSolve(LagRBFCtx ctx, Partition p, PetscInt nfields, PetscReal *data) { return 0; }
PetscErrorCode LagRBFGPU_PartitionDestroy(Partition p) { return 0; }

/* A swarm's coordinates, pids and (nullable) named field, borrowed from the DMSwarm. */
typedef struct {
  DM sw;
  PetscInt n, bs;
  const char *cname, *fname;
  PetscReal *x, *f;
  PetscInt64 *pid;
} swarm_view;

static PetscErrorCode view_get(DM sw, const char *fname, swarm_view *v)
{
  DMSwarmCellDM celldm;
  const char **cn;
  PetscErrorCode e;
  memset(v, 0, sizeof(*v));
  v->sw = sw;
  v->fname = fname;
  if ((e = DMSwarmGetLocalSize(sw, &v->n))) return e;
  if ((e = DMSwarmGetCellDMActive(sw, &celldm))) return e;
  if ((e = DMSwarmCellDMGetCoordinateFields(celldm, NULL, &cn))) return e;
  v->cname = cn[0];
  if ((e = DMSwarmGetField(sw, v->cname, NULL, NULL, (void **)&v->x))) return e;
  if ((e = DMSwarmGetField(sw, DMSwarmField_pid, NULL, NULL, (void **)&v->pid))) return e;
  if (fname && (e = DMSwarmGetField(sw, fname, &v->bs, NULL, (void **)&v->f))) return e;
  return 0;
}

static PetscErrorCode view_restore(swarm_view *v)
{
  PetscErrorCode e;
  if (v->fname && (e = DMSwarmRestoreField(v->sw, v->fname, &v->bs, NULL, (void **)&v->f))) return e;
  if ((e = DMSwarmRestoreField(v->sw, DMSwarmField_pid, NULL, NULL, (void **)&v->pid))) return e;
  return DMSwarmRestoreField(v->sw, v->cname, NULL, NULL, (void **)&v->x);
}

static PetscInt64 max_pid(const swarm_view *v)
{
  PetscInt64 m = 0;
  PetscInt p;
  for (p = 0; p < v->n; p++) m = v->pid[p] > m ? v->pid[p] : m;
  return m;
}

/* Data swarm and particle swarm into the GPU context (the data's unchanged coordinates keep their
   binning and factors); the particles' "fields" go in as their current values. */
static PetscErrorCode fill_both(LagRBFCtx ctx, void *gpu, DM swi, DM swd, int with_fields)
{
  swarm_view d, i;
  PetscErrorCode e;
  if ((e = view_get(swd, "fields", &d))) return e;
  e = lagrbf_fill_swarm(gpu, true, d.n, d.x, d.f, d.pid);
  view_restore(&d);
  if (e) return e;
  if ((e = view_get(swi, with_fields ? "fields" : NULL, &i))) return e;
  e = lagrbf_fill_swarm(gpu, false, i.n, i.x, with_fields ? i.f : NULL, i.pid);
  view_restore(&i);
  return e;
}

/* rows[pid - 1] of an output of nglobal rows x bs into the swarm field, in swarm order */
static void rows_to_swarm(const swarm_view *v, const double *rows, int bs_rows, double *dst, int bs)
{
  PetscInt p;
  int k;
  for (p = 0; p < v->n; p++)
    if (v->pid[p] > 0)
      for (k = 0; k < bs; k++) dst[(size_t)p * bs + k] = rows[(size_t)(v->pid[p] - 1) * bs_rows + k];
}

PetscErrorCode LagRBFGPU_RBFInterpolation(LagRBFCtx ctx, DM swi, DM swd, const char *fieldname)
{
  void *gpu = gpu_of(ctx);
  swarm_view v;
  PetscErrorCode e;
  PetscInt64 ng;
  double *rows;
  int F = (int)ctx->n_ifields;
  if (!gpu) return LAGRBF_ERR_ARG_WRONGSTATE;
  if ((e = fill_both(ctx, gpu, swi, swd, 0))) return e;
  if ((e = lagrbf_interpolation(gpu))) return e;
  if ((e = view_get(swi, fieldname, &v))) return e;
  ng = max_pid(&v);
  rows = (double *)calloc((size_t)(ng > 0 ? ng : 1) * (size_t)(F > 0 ? F : 1), sizeof(double));
  if (!rows) { view_restore(&v); return LAGRBF_ERR_MEM; }
  /* the interpolated fields; a "velocity" target takes their first dim components */
  e = lagrbf_output(gpu, false, (int32_t)ng, NULL, rows, NULL, "fields");
  if (!e) rows_to_swarm(&v, rows, F, v.f, (int)(v.bs < F ? v.bs : F));
  free(rows);
  view_restore(&v);
  return e;
}

PetscErrorCode LagRBFGPU_SwarmInterpSetWeights(LagRBFCtx ctx, DM sw)
{
  void *gpu = gpu_of(ctx);
  swarm_view v;
  PetscErrorCode e;
  PetscInt64 ng;
  double *rows;
  int nen = 1 << ctx->pu->dim;
  if (!gpu) return LAGRBF_ERR_ARG_WRONGSTATE;
  if ((e = view_get(sw, "weights", &v))) return e;
  e = lagrbf_fill_swarm(gpu, false, v.n, v.x, NULL, v.pid);
  ng = max_pid(&v);
  rows = (double *)calloc((size_t)(ng > 0 ? ng : 1) * (size_t)nen, sizeof(double));
  if (!e && !rows) e = LAGRBF_ERR_MEM;
  if (!e) e = lagrbf_output(gpu, false, (int32_t)ng, NULL, rows, NULL, "weights");
  if (!e) rows_to_swarm(&v, rows, nen, v.f, nen);
  free(rows);
  view_restore(&v);
  return e;
}

/* One internal step of size adv_ctx->dt (the caller's time loop has already limited it by the
   CFL condition, which the GPU computes identically, so it takes a single step): positions,
   "fields" and "velocity" written back by pid; particles that left the domain are removed from
   the swarm, as DMSwarmMigrate removes them on one rank. */
PetscErrorCode LagRBFGPU_AdvectionStep(LagRBFCtx ctx, DM swi, DM swd)
{
  void *gpu = gpu_of(ctx);
  swarm_view v;
  PetscErrorCode e;
  PetscInt64 ng;
  PetscInt p;
  double *x, *f;
  int64_t *pid;
  int dim = (int)ctx->pu->dim, F = (int)ctx->n_ifields;
  if (!gpu) return LAGRBF_ERR_ARG_WRONGSTATE;
  if ((e = fill_both(ctx, gpu, swi, swd, 1))) return e;
  if ((e = lagrbf_gpu_advect_resident(gpu, 0.0, ctx->adv_ctx->dt))) return e;
  if ((e = view_get(swi, "fields", &v))) return e;
  ng = max_pid(&v);
  x = (double *)calloc((size_t)(ng > 0 ? ng : 1) * (size_t)dim, sizeof(double));
  f = (double *)calloc((size_t)(ng > 0 ? ng : 1) * (size_t)(F > 0 ? F : 1), sizeof(double));
  pid = (int64_t *)calloc((size_t)(ng > 0 ? ng : 1), sizeof(int64_t));
  e = (!x || !f || !pid) ? LAGRBF_ERR_MEM : lagrbf_output(gpu, false, (int32_t)ng, x, f, pid, "fields");
  if (!e) {
    double *vel = NULL;
    rows_to_swarm(&v, x, dim, v.x, dim);
    rows_to_swarm(&v, f, F, v.f, F);
    if (!DMSwarmGetField(swi, "velocity", NULL, NULL, (void **)&vel)) {
      rows_to_swarm(&v, f, F, vel, dim < F ? dim : F);
      DMSwarmRestoreField(swi, "velocity", NULL, NULL, (void **)&vel);
    }
  }
  view_restore(&v);
  /* removed particles: their pid rows came back zero; delete from the end so indices hold */
  for (p = v.n - 1; !e && p >= 0; p--) {
    PetscInt64 id = 0;
    PetscInt64 *pp;
    if (DMSwarmGetField(swi, DMSwarmField_pid, NULL, NULL, (void **)&pp)) break;
    id = pp[p];
    DMSwarmRestoreField(swi, DMSwarmField_pid, NULL, NULL, (void **)&pp);
    if (id > 0 && id <= ng && pid[id - 1] == 0) e = DMSwarmRemovePointAtIndex(swi, p);
  }
  free(x); free(f); free(pid);
  return e;
}

#if defined(LAGRBF_GPU_REPLACE)
/* The reference names, for builds that leave out interpolation.c's RBFInterpolation and
   swarm_interp.c's SwarmInterpSetWeights dispatcher. */
PetscErrorCode RBFInterpolation(LagRBFCtx ctx, DM swi, DM swd, const char *fieldname)
{
  return LagRBFGPU_RBFInterpolation(ctx, swi, swd, fieldname);
}
PetscErrorCode SwarmInterpSetWeights(LagRBFCtx ctx, DM sw) { return LagRBFGPU_SwarmInterpSetWeights(ctx, sw); }
#endif
