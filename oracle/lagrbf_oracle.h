/*
 * lagrbf_oracle.h -- CPU restatement of LagRBF's PU-RBF interpolation and advection path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the parity checker for the GB300 implementation
 * in lagrbf_gb300/.  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may
 * load it.  The product never links against it and never falls back to it.
 *
 * Parity status: parity unpinned.  The reference ships no assertion-based tests and no golden
 * vectors for this path, and it cannot be built here as shipped (it needs PETSc).  Where the
 * reference delegates to PETSc (point location, per-cell point order, Q1 element node order,
 * LAPACK Cholesky), this restatement fixes the convention documented next to each function.
 *
 * Every function cites the reference file:line it restates.
 */
#ifndef LAGRBF_ORACLE_H
#define LAGRBF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* KernelType order of include/kernels/kernels_rbf.h:34-42 */
enum { ORC_KERNEL_LINEAR = 0, ORC_KERNEL_WENDLAND_C0, ORC_KERNEL_WENDLAND_C2, ORC_KERNEL_BUMP,
       ORC_KERNEL_MQ, ORC_KERNEL_IMQ, ORC_KERNEL_GAUSSIAN };
/* ASolveMethod of include/lagrangian_rbf.h (A_FACTOR, A_KSP, A_KSP_ASMB) */
enum { ORC_A_FACTOR = 0, ORC_A_KSP = 1, ORC_A_KSP_ASMB = 2 };
/* AdvectionScheme of include/advection/advection_ctx.h:34-39 */
enum { ORC_RK1 = 0, ORC_RK2 = 1, ORC_RK4 = 2, ORC_DOPRI = 3 };

typedef struct {
  int    dim;          /* pu_mesh_dim                                            */
  int    n[3];         /* pu_mesh_n: nodes (= patches) per dimension              */
  double O[3], L[3];   /* pu_mesh_O / pu_mesh_L                                    */
  double overlap;      /* pu_mesh_overlap                                         */
  double shape_factor; /* pu_mesh_shape_factor                                    */
  int    kernel;       /* kernel_type                                             */
  int    solve_method; /* solve_method                                            */
  int    nfields;      /* n_interpolation_fields                                  */
  int    advection;    /* advection (bool)                                        */
  int    scheme;       /* advection_scheme                                        */
  double cfl_fac, dt, rmin, rmax;
  double dopri_dt_fac, dopri_dt_fac_min, dopri_dt_fac_max, dopri_atol, dopri_rtol;
  int    dopri_per_particle; /* extension: per-particle adaptive Dormand-Prince (0: the reference's
                                single global step, always accepted)                              */
  int    setup_all;          /* extension: set up every patch, not only those of cells holding
                                particles (the lazy set-up of partition.c:452-469)               */
} orc_config;

/* Defaults of LagRBFCtxCreate (src/lagrangian_rbf.c:36-73), AdvectionCtxCreate
   (src/advection/advection_ctx.c:52-65) and DOPRICtxCreate (src/advection/dormand_prince.c:312-327). */
void orc_config_default(orc_config *cfg);

/* ---------------- geometry and kernels ---------------- */
typedef struct {
  int    dim, n[3], nnodes, ncells, nen;
  double O[3], L[3], h[3];
  double eps_w, eps_r;
} orc_pu;

/* partition_of_unity.c:322-355 (support and shape factor), :143 (uniform node coordinates) */
void   orc_pu_setup(orc_pu *pu, const orc_config *cfg);
/* kernels_rbf.c:31-91 */
double orc_phi_scalar(int kernel, double r, double eps);
/* One lane of the vector kernels (kernels_rbf_avx512.h:34-95, kernels_rbf_avx.h:35-94 op order). */
double orc_phi_lane(int kernel, double r, double eps);
/* Q1 corner k of cell `cell` (PETSc DMDAGetElements node order). */
int    orc_cell_corner(const orc_pu *pu, int cell, int k);

/* ---------------- binning (a2, a3, a4) ---------------- */
/* Cell id per point; -1 when the point lies outside [O,L] (DMSwarmPICSetCellId, swarm_utils.c:995-1029). */
void orc_locate(const orc_pu *pu, int np, const double *coords, int *cellid);
/* Counting sort by cell, stable in point index (DMSwarmSortGetAccess / GetPointsPerCell). */
void orc_cell_csr(const orc_pu *pu, int np, const int *cellid, int *cell_start, int *cell_pts);
/* Patch membership: partition.c:54-87 (inverse map) and :337-371 (concatenation).  Returns sum of sizes
   when patch_pts == NULL. */
long orc_patch_csr(const orc_pu *pu, const int *cell_start, const int *cell_pts, int *patch_start, int *patch_pts);
/* 3^dim evaluation block: cell_info.c:120-297 (neighbour order) and :468-501. */
long orc_block_csr(const orc_pu *pu, const int *cell_start, const int *cell_pts, int *blk_start, int *blk_pts);

/* ---------------- weights (a5) ---------------- */
/* SwarmInterpSetWeights_AVX256, weights_avx.c:97-243 (sum over every node, groups of 4). */
void orc_weights(const orc_pu *pu, int np, const double *coords, const int *cellid, const int *alive,
                 double *weights);

/* ---------------- patch solve (a6, a7) ---------------- */
/* Assemble (partition_asmb_avx512.c:119-198), Cholesky (LAPACK potrf semantics) and solve
   (partition_factor.c:57-135).  coeffs is column-major [f*m + j].  Returns 0, or the 1-based
   row of a non-positive pivot. */
void orc_assemble(const orc_pu *pu, int kernel, int m, const int *idx, const double *coords, double *A);
int orc_patch_solve(const orc_pu *pu, int kernel, int m, const int *idx, const double *coords,
                    int nfields, const double *values, double *coeffs);

/* ---------------- evaluation (a8) ---------------- */
/* PointwiseInterpolation_AVX512, interpolation_avx512.c:121-291.  coeffs[k] (NULL = patch not set up)
   holds column-major coefficients of patch k with leading dimension m_k = patch size;
   nf is the block size of the target field (its first nf coefficient columns are used). */
void orc_eval(const orc_pu *pu, int kernel, int np, const double *xp, const int *cellid, const int *alive,
              const double *weights, const double *xd, const int *blk_start, const int *blk_pts,
              const int *patch_start, const int *patch_pts, const int *patch_setup, double *const *coeffs,
              int nf, double *values);

/* ---------------- reference-API emulation ---------------- */
typedef struct orc_ctx orc_ctx;
/* Accepted particle steps of per-particle Dormand-Prince since the context was created. */
long long orc_get_accepted(orc_ctx *c);
typedef int (*orc_velocity_fn)(double *coords, double *velocity, void *user);
typedef int (*orc_velocity_batch_fn)(int32_t npoints, int32_t dim, double *coords, double *velocity, void *user);

orc_ctx *orc_create(const orc_config *cfg);                                   /* interface_ctx.c:54-104 */
void     orc_destroy(orc_ctx *ctx);
int      orc_fill_swarm(orc_ctx *ctx, int is_data, int n, const double *coords, const double *values,
                        const int64_t *pidx);                                  /* interface_utils.c:68-165 */
int      orc_interpolation(orc_ctx *ctx);                                     /* interface_interp.c:83-96 */
int      orc_output(orc_ctx *ctx, int is_data, int nglobal, double *coords, double *fields, int64_t *pidx,
                    const char *fieldname);                                   /* interface_utils.c:188-339 */
int      orc_reset_coefficients(orc_ctx *ctx);                                /* partition.c:494-524 */
int      orc_advect_interpolate(orc_ctx *ctx, double t, double t_next);      /* time_loop.c:39-100 */
int      orc_advect_analytical(orc_ctx *ctx, double t, double t_next);       /* time_loop.c:176-221 */
int      orc_set_velocity_fn(orc_ctx *ctx, orc_velocity_fn fn, void *user);
int      orc_set_velocity_batch_fn(orc_ctx *ctx, orc_velocity_batch_fn fn, void *user);
/* Coupling of sharded runs (the reference's MPI_Allreduce at advection.c:466 and
   dormand_prince.c:93): fn replaces vals[0..n) by their element-wise maximum over the ranks.  Each
   internal step the oracle passes {-(CFL step), DOPRI error} (the negated step, so that the maximum
   is the global minimum step). */
typedef int (*orc_step_reduce_fn)(double *vals, int32_t n, void *user);
int      orc_set_step_reduce(orc_ctx *ctx, orc_step_reduce_fn fn, void *user);
/* Inspection for tests. */
int      orc_get_counts(orc_ctx *ctx, int *nd, int *np_alive, int *npatch_setup, int *nsteps);
double   orc_get_dt(orc_ctx *ctx);
int      orc_get_cellids(orc_ctx *ctx, int is_data, int *cellid);
long     orc_get_patch_csr(orc_ctx *ctx, int *patch_start, int *patch_pts);
long     orc_get_block_csr(orc_ctx *ctx, int *blk_start, int *blk_pts);
int      orc_get_weights(orc_ctx *ctx, double *weights);

/* Multi-threaded timing leg for the CPU baseline: the whole-dataset patch setup plus `nsteps`
   calls of advect_interpolate over [t, t+dt] on a particle sample, one OpenMP thread per
   emulated MPI rank (disjoint particle subsets, replicated patches).  Returns seconds of the
   stepping loop in *step_s and of the setup in *setup_s. */
int      orc_time_baseline(const orc_config *cfg, int nd, const double *xd, const double *fd, int np,
                           const double *xp, int nsteps, double dt, int nthreads, double *setup_s,
                           double *step_s);

/* Emulated MPI ranks, each its own sub-problem (local PU sub-mesh with halo, the data of its
   local box, a particle sample): one OpenMP thread per rank, setup then `nsteps` steady-state
   advection steps of [t, t+dt].  Returns live particle-steps advanced in *psteps. */
int      orc_time_ranks(int nranks, const orc_config *cfgs, const int *nd, const double *const *xd,
                        const double *const *fd, const int *np, const double *const *xp, int nsteps, double dt,
                        double *setup_s, double *step_s, long *psteps);

#ifdef __cplusplus
}
#endif
#endif
