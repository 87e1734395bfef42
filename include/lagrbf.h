/*
 * lagrbf.h -- C-ABI of the GB300 implementation of LagRBF's PU-RBF interpolation and advection
 * path (liblagrbf.so in lagrbf_gb300/).
 *
 * Section 1 is the drop-in surface: the same eleven exported symbols, argument meaning and
 * error behaviour as LagRBF's ctypes interface (python_api/lagrbfpy/interface/register_cfunc.py:
 * 50-191; implementations in the src/interface/ C files).  PetscInt is int32_t, PetscReal is double,
 * PetscInt64 is int64_t and PetscErrorCode is int (0 = success).  `is_data` is declared bool,
 * which is how the ctypes binding passes it (register_cfunc.py:95,118).
 *
 * Section 2 replaces the PETSc options database that lagrbf_create() reads
 * (LagRBFSetFromOptions, src/lagrangian_rbf.c:135-195; PUSetFromOptions,
 * src/partition_of_unity.c:68-111; DOPRICtxSetFromOptions, src/advection/dormand_prince.c:340-353).
 * Keys are the PETSc option names without the leading dash.
 *
 * Section 3 is the GPU-level extension used by the benchmark, the tests and the serving loop.
 * It has no counterpart in the reference.
 *
 * Error codes follow PETSc's numbering for the analogous failures; LAGRBF_ERR_* below.
 * No function aborts, traps or exits the process.
 */
#ifndef LAGRBF_GB300_H
#define LAGRBF_GB300_H

#include <stdbool.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define LAGRBF_EXPORT __attribute__((visibility("default")))

enum {
  LAGRBF_SUCCESS = 0,
  LAGRBF_ERR_MEM = 55,            /* device or host allocation failed                     */
  LAGRBF_ERR_SUP = 56,            /* option value not supported                            */
  LAGRBF_ERR_ARG_SIZ = 60,        /* inconsistent sizes                                    */
  LAGRBF_ERR_ARG_WRONG = 62,      /* e.g. a point outside the PU bounding box on fill      */
  LAGRBF_ERR_ARG_OUTOFRANGE = 63, /* e.g. a pid outside [1, npoints] on output             */
  LAGRBF_ERR_ARG_WRONGSTATE = 73, /* call order violated (data not filled, ...)            */
  LAGRBF_ERR_PLIB = 77,           /* internal inconsistency                                */
  LAGRBF_ERR_MAT_CH_ZRPVT = 81,   /* non-positive pivot in a patch Cholesky factorisation  */
  LAGRBF_ERR_ARG_NULL = 85,       /* NULL context / array                                  */
  LAGRBF_ERR_GPU = 97,            /* CUDA runtime error                                    */
  LAGRBF_ERR_TIMEOUT = 200        /* a bounded device wait gave up                         */
};

/* ---------------------------------------------------------------------------------------- */
/* 1. Drop-in surface (LagRBF ctypes interface)                                              */
/* ---------------------------------------------------------------------------------------- */

/* Replaces lagrbf_create, src/interface/interface_ctx.c:93-104 (NULL on error). */
LAGRBF_EXPORT void *lagrbf_create(void);
/* Replaces lagrbf_destroy, src/interface/interface_ctx.c:120-125. */
LAGRBF_EXPORT void lagrbf_destroy(void *ctx);
/* Replaces lagrbf_fill_swarm, src/interface/interface_utils.c:403-430.  coords is n*dim,
   values (nullable) is n*n_interpolation_fields, pidx (nullable) holds 1-based unique ids. */
LAGRBF_EXPORT int lagrbf_fill_swarm(void *ctx, bool is_data, int32_t npoints, double *coords, double *values,
                                    int64_t *pidx);
/* Replaces lagrbf_interpolation, src/interface/interface_interp.c:210-221. */
LAGRBF_EXPORT int lagrbf_interpolation(void *ctx);
/* Replaces lagrbf_output, src/interface/interface_utils.c:362-384.  Outputs are caller-allocated,
   npoints rows, assembled by pid-1; rows of points no longer in the swarm are zero. */
LAGRBF_EXPORT int lagrbf_output(void *ctx, bool is_data, int32_t npoints, double *coords, double *fields,
                                int64_t *pidx, const char *fieldname);
/* Replaces lagrbf_reset_coefficients, src/interface/interface_utils.c:447-458. */
LAGRBF_EXPORT int lagrbf_reset_coefficients(void *ctx);
/* Replaces lagrbf_avect_analytical, src/interface/interface_adv.c:75-88. */
LAGRBF_EXPORT int lagrbf_avect_analytical(void *ctx, double time, double time_next);
/* Replaces lagrbf_advect_interpolate, src/interface/interface_adv.c:90-106 (registered in Python
   under the key "lagrbf_avect_interpolate"). */
LAGRBF_EXPORT int lagrbf_advect_interpolate(void *ctx, double time, double time_next);
/* Replaces lagrbf_advection_function, src/interface/interface_adv.c:35-53. */
LAGRBF_EXPORT int lagrbf_advection_function(void *ctx, int (*velocity_fn)(double *, double *, void *), void *fn_ctx);
/* Replaces lagrbf_advection_function_batch, src/interface/interface_adv.c:55-73. */
LAGRBF_EXPORT int lagrbf_advection_function_batch(void *ctx,
                                                  int (*velocity_fn_batch)(int32_t, int32_t, double *, double *, void *),
                                                  void *fn_ctx);
/* Replaces lagrbf_interpolate_driver, src/interface/interface_interp.c:167-194.  options_file
   (nullable) uses PETSc's options-file syntax: "-key value" pairs, '#' comments. */
LAGRBF_EXPORT void lagrbf_interpolate_driver(int32_t ndata_local, double *data_coords, double *data_values,
                                             int32_t npoints_local, double *points_coords, double *points_values,
                                             int32_t npoints_global, char *options_file);

/* ---------------------------------------------------------------------------------------- */
/* 2. Options store (stands in for PetscOptionsSetValue / PetscOptionsInsertFile)            */
/* ---------------------------------------------------------------------------------------- */
/* Keys read by lagrbf_create(): pu_mesh_dim, pu_mesh_n, pu_mesh_O, pu_mesh_L, pu_mesh_overlap,
   pu_mesh_shape_factor, n_interpolation_fields, kernel_type, solve_method, advection,
   advection_scheme, velocity_name, dt, cfl_fac, rmin, rmax, dopri_dt_fac, dopri_dt_fac_min,
   dopri_dt_fac_max, dopri_atol, dopri_rtol; and the GPU-only keys eval_precision (fp64|fp32,
   default fp64), use_cuda_graph (bool, default true), device_loop (bool, default true: an
   advection interval runs as one graph launch whose step is the body of a device-side while loop;
   false keeps one graph launch per internal step, whose kernels profilers can attribute),
   cuda_device (int), output_direct (bool,
   default true: when the device accesses pageable host memory, lagrbf_output's particle rows are
   written by the GPU straight into the caller's arrays and lagrbf_fill_swarm's data arrays are
   read by it directly), dopri_per_particle (bool, default false: per-particle adaptive
   Dormand-Prince, an extension), setup_all_patches (bool, default false: set up every patch, not
   only those of cells holding particles).  Arrays are comma separated. */
LAGRBF_EXPORT int lagrbf_options_set_value(const char *name, const char *value);
LAGRBF_EXPORT int lagrbf_options_clear(void);
LAGRBF_EXPORT int lagrbf_options_insert_file(const char *path);
/* Copies the stored value into buf; returns 1 if found, 0 if not. */
LAGRBF_EXPORT int lagrbf_options_get_value(const char *name, char *buf, int32_t buflen);

/* ---------------------------------------------------------------------------------------- */
/* 3. GPU-level extension (no counterpart in the reference)                                  */
/* ---------------------------------------------------------------------------------------- */
typedef struct {
  int64_t launches;           /* kernels this context launched (graph nodes counted)          */
  int64_t eval_launches;      /* launches of the PU evaluation kernel                        */
  double  eval_flops;         /* algorithmic flops of those launches (counted on the device) */
  double  eval_bytes;         /* algorithmic bytes of those launches                         */
  double  eval_ms;            /* event-timed duration of those launches (profiling on)       */
  int64_t particle_steps;     /* live particles x internal steps advanced                     */
  int64_t steps;              /* internal time steps taken                                   */
  int64_t patches_factored;   /* patch Cholesky factorisations performed                     */
  double  factor_ms;          /* event-timed factorisation time (profiling on)               */
  double  factor_flops;       /* algorithmic flops of those factorisations                   */
  int32_t np_alive;           /* particles still in the swarm                                */
  int32_t nd;                 /* data points in the swarm                                    */
  int32_t max_patch;          /* largest patch (data points)                                 */
  int32_t npatch_setup;       /* patches currently set up                                    */
  double  dt;                 /* the advection context's current time step                   */
  int32_t chunk_cap;          /* particles per evaluation work unit                          */
  int32_t records;            /* 1 when precomputed record blocks are streamed by TMA         */
  double  kappa_max;          /* largest / median 1-norm condition estimate of the patches     */
  double  kappa_median;       /* factored with lagrbf_gpu_set_condition_estimates on (else 0)  */
  int32_t device_loop;        /* 1 when advection intervals run as one graph launch with the
                                 internal steps looping on the device (conditional while node)  */
} lagrbf_stats_t;

/* The interpolated advection loop of lagrbf_advect_interpolate over [time, time_next] without its
   end-of-call reset: the data swarm, binning and patch set-ups stay resident for the next call. */
LAGRBF_EXPORT int lagrbf_gpu_advect_resident(void *ctx, double time, double time_next);
/* Device-side analytical velocity for lagrbf_avect_analytical (replaces the per-stage host
   callback round trip of lagrbf_advection_function(_batch); takes precedence over a registered
   callback; kind 0 removes it).  Parameters:
     LAGRBF_VFIELD_ROTATION {omega, cx, cy}:  v = omega (-(y - cy), x - cx, 0)
     LAGRBF_VFIELD_CELLULAR {a, k}:           v = a (sin(k pi x) cos(k pi y), -cos(k pi x) sin(k pi y), 0)
     LAGRBF_VFIELD_ABC      {A, B, C, s}:     X = s x: (A sin Z + C cos Y, B sin X + A cos Z, C sin Y + B cos X)
     LAGRBF_VFIELD_FOURIER  {n, n x (k1, k2, k3, phase, a1, a2, a3)}: v_c = sum_m a_mc sin(2 pi k_m.x + phase_m) */
enum { LAGRBF_VFIELD_NONE = 0, LAGRBF_VFIELD_ROTATION = 1, LAGRBF_VFIELD_CELLULAR = 2, LAGRBF_VFIELD_ABC = 3,
       LAGRBF_VFIELD_FOURIER = 4 };
LAGRBF_EXPORT int lagrbf_gpu_set_velocity_field(void *ctx, int32_t kind, const double *params, int32_t nparams);
/* Switches the evaluation precision of a live context (1: FP32 evaluation, 0: FP64). */
LAGRBF_EXPORT int lagrbf_gpu_set_precision(void *ctx, int fp32);
/* FP32 FMA throughput of the current device in TFLOP/s, measured by a synthetic kernel
   (dependent FFMA chains, all SMs): the FP32 roofline denominator. */
LAGRBF_EXPORT double lagrbf_gpu_fp32_peak_tflops(void);
/* The same for FP64 (dependent DFMA chains): the FP64 roofline denominator. */
LAGRBF_EXPORT double lagrbf_gpu_fp64_peak_tflops(void);
/* Per-patch condition estimates: while on, every patch factorisation also estimates
   kappa_1(A) = ||A||_1 ||A^-1||_1 of its collocation matrix (||A^-1||_1 by Hager's method as refined
   by Higham, a few extra triangular solves per patch; the factorisation itself is unchanged).
   lagrbf_gpu_get_condition copies the estimates by node (kappa, nullable, nnodes entries, 0 for
   patches not factored while on) and summary[3] = {max, median, count} of the non-zero ones. */
LAGRBF_EXPORT int lagrbf_gpu_set_condition_estimates(void *ctx, int on);
LAGRBF_EXPORT int lagrbf_gpu_get_condition(void *ctx, double *kappa, double *summary);
/* Several particle sets on one resident dataset, concurrently: ctx (a fresh context with the same
   options, no data of its own) uses owner's data swarm, patch set-ups, coefficients, factors and
   record blocks in place, read-only, on its own stream with its own particles.  The owner needs the
   option setup_all_patches and a completed interpolation (every patch set up and solved), so that
   nothing ctx does writes the shared state; lagrbf_fill_swarm of the data on ctx is refused and its
   coefficient reset does nothing.  The owner must outlive ctx and keep its data unchanged while ctx
   is in use.  The call does not touch the owner's stream, so the owner's thread may go on
   advecting its own particles meanwhile (its interpolation must have returned before this call,
   ordered by the caller's own thread synchronisation). */
LAGRBF_EXPORT int lagrbf_gpu_share_dataset(void *ctx, void *owner);
/* Coupling of sharded runs (one process and GPU per rank, each holding the whole dataset and a pid
   range of the particles): fn(vals, n, user) must replace vals[0..n) by their element-wise maximum
   over the ranks (e.g. an MPI_Allreduce with MPI_MAX) and return 0.  Each internal step of the
   advection loops passes {-(the local CFL step), the local Dormand-Prince error}, so every rank takes
   the reference's global step (advection.c:466, dormand_prince.c:93) for any outer interval, and
   once before the first step.  Per-particle Dormand-Prince needs no coupling and does not call it.
   The reference sets up only the patches of cells holding particles (partition.c:452-469), which
   depends on where every rank's particles are: sharded runs equal the single-rank run bit for bit
   when both use the option setup_all_patches (every patch set up).  NULL removes it. */
LAGRBF_EXPORT int lagrbf_gpu_set_step_reduce(void *ctx, int (*fn)(double *vals, int32_t n, void *user), void *user);
/* Test hook of the evaluation kernel's bounded waits: poll_limit (> 0) replaces the default number
   of polls after which a wait on a staging copy gives up (0 restores it); with withhold_copies the
   kernel arms its staging barriers but issues no copy, so every wait runs out and the call returns
   LAGRBF_ERR_TIMEOUT with the context still usable.  Applies to the FP32 evaluation of the velocity
   fields from record blocks (the path of lagrbf_gpu_set_precision(ctx, 1) with F >= dim). */
LAGRBF_EXPORT int lagrbf_gpu_test_eval_wait(void *ctx, int32_t poll_limit, int32_t withhold_copies);
/* Kernel-level event timing of the evaluation and factorisation launches (disables graph
   capture while on, so every launch is bracketed by events on the context's stream). */
LAGRBF_EXPORT int lagrbf_gpu_set_profiling(void *ctx, int on);
LAGRBF_EXPORT int lagrbf_gpu_get_stats(void *ctx, lagrbf_stats_t *stats);
LAGRBF_EXPORT int lagrbf_gpu_reset_stats(void *ctx);
/* Blocks until all work of the context is done. */
LAGRBF_EXPORT int lagrbf_gpu_synchronize(void *ctx);
/* The context's cudaStream_t, as void*. */
LAGRBF_EXPORT void *lagrbf_gpu_stream(void *ctx);
/* Last error message of the calling thread (empty string if none). */
LAGRBF_EXPORT const char *lagrbf_gpu_last_error(void);
/* Per-cell/per-patch views for parity tests (host arrays sized by the caller):
   cellid[n] of the data (is_data) or particle swarm; cell_start[ncells+1] and the data points of
   each cell in order; patch_start[nnodes+1] and patch_pts[] (data indices, reference order). */
LAGRBF_EXPORT int lagrbf_gpu_get_cellids(void *ctx, bool is_data, int32_t *cellid);
LAGRBF_EXPORT int64_t lagrbf_gpu_get_patch_csr(void *ctx, int32_t *patch_start, int32_t *patch_pts);
LAGRBF_EXPORT int64_t lagrbf_gpu_get_block_csr(void *ctx, int32_t *blk_start, int32_t *blk_pts);
/* Geometry of the context: dim, n[3], nnodes, ncells, nen and eps_w, eps_r. */
LAGRBF_EXPORT int lagrbf_gpu_get_geometry(void *ctx, int32_t *ints /* 7 */, double *reals /* 2 */);

/* ---------------------------------------------------------------------------------------- */
/* 4. PETSc binary files (no PETSc needed)                                                   */
/* ---------------------------------------------------------------------------------------- */
/* PETSc binary viewer format, 32-bit PetscInt, big-endian: Vec = class id 1211214, n, n doubles;
   IS = class id 1211218, n, n int32.  A Vec's block size is read from / written to "<path>.info"
   ("-vecload_block_size <bs>").  Readers: pass NULL for the buffer to get the length first.
   Replace VecLoadFromFile / ISLoadFromFile (src/io_utils.c:211-238) and the VecView / ISView
   writers of src/swarm/swarm_output.c:87-166. */
LAGRBF_EXPORT int lagrbf_petsc_vec_write(const char *path, const double *values, int64_t n, int32_t block_size);
LAGRBF_EXPORT int lagrbf_petsc_vec_read(const char *path, double *values, int64_t capacity, int64_t *n,
                                        int32_t *block_size);
LAGRBF_EXPORT int lagrbf_petsc_is_write(const char *path, const int64_t *indices, int64_t n);
LAGRBF_EXPORT int lagrbf_petsc_is_read(const char *path, int64_t *indices, int64_t capacity, int64_t *n);
/* SwarmSetFromPetscFiles (src/readers/petsc_loader/petsc_loader.c:38-99): coordinates from
   coords_file (block size dim) set the number of points; the field files fill
   n_interpolation_fields in file order by block; pid_file (nullable, an IS) gives the pids
   (SwarmInterpLoadPidxFromFile, src/swarm/swarm_interp.c:180-222).  Then lagrbf_fill_swarm. */
LAGRBF_EXPORT int lagrbf_fill_swarm_from_files(void *ctx, bool is_data, const char *coords_file,
                                               const char **field_files, int32_t nfiles, const char *pid_file);
/* lagrbf_output into files: <prefix>_coor.pbvec, <prefix>_<fieldname>.pbvec (with .info) and
   <prefix>_pid.pbis, nglobal rows assembled by pid. */
LAGRBF_EXPORT int lagrbf_output_files(void *ctx, bool is_data, int32_t nglobal, const char *prefix,
                                      const char *fieldname);

/* ---------------------------------------------------------------------------------------- */
/* 5. Serving loop (no counterpart in the reference)                                          */
/* ---------------------------------------------------------------------------------------- */
/* An advection job: the PU mesh and kernel of its dataset, the dataset itself (nd points, nfields
   values each) or the id of a resident one, nsteps steps of size dt of the RK scheme
   (0 RK1, 1 RK2, 2 RK4, 3 Dormand-Prince; CFL-limited inside each step like
   lagrbf_advect_interpolate) on np particles.  Inputs are copied at submission. */
typedef struct {
  int32_t dim, nodes[3];
  double O[3], L[3], overlap, shape_factor;
  int32_t kernel, nfields;
  int64_t dataset_id;     /* > 0: kept resident after the job under this id; 0: private */
  int32_t nd;
  const double *data_coords, *data_values; /* NULL for a resident dataset id */
  int32_t np;
  const double *particles;
  int32_t scheme, nsteps;
  double dt, cfl;          /* cfl <= 0: 0.3 */
  int32_t fp32;            /* 1: FP32 evaluation */
} lagrbf_job_t;
typedef struct {
  int64_t submitted, completed, failed, queued, running;
  double p50_ms, p99_ms, mean_ms, max_ms; /* submission-to-completion latency of completed jobs */
  double particle_steps, elapsed_s, bytes_in_use;
  int32_t datasets_resident;
  double queue_p50_ms, queue_p99_ms;      /* submission to start (waiting in the queue)          */
  double service_p50_ms, service_p99_ms;  /* start to completion (set-up if any, steps, output)  */
} lagrbf_server_stats_t;
/* Worker threads (one context and CUDA stream per running job) admit queued jobs first in, first
   out as the device-memory budget and their dataset allow; a job may pass a waiting one that does
   not fit yet, unless that one has waited over two seconds.  Idle resident datasets are evicted
   least recently used first.  Latency is measured from submission. */
LAGRBF_EXPORT void *lagrbf_server_create(double hbm_budget_bytes, int32_t nworkers);
LAGRBF_EXPORT int lagrbf_server_submit(void *server, const lagrbf_job_t *job, int64_t *job_id);
/* Blocks until the job is done; positions (nullable, np*dim) receive its particles by pid (rows of
   particles that left the domain are zero). */
LAGRBF_EXPORT int lagrbf_server_wait(void *server, int64_t job_id, double *positions, double *latency_ms);
LAGRBF_EXPORT int lagrbf_server_stats(void *server, lagrbf_server_stats_t *stats);
LAGRBF_EXPORT int lagrbf_server_reset_stats(void *server);
/* Cancels queued jobs, lets running ones finish, frees every resident dataset. */
LAGRBF_EXPORT void lagrbf_server_destroy(void *server);

/* Binning without device allocation (no counterpart in the reference).  For callers that may not
   have a library allocate device memory at this point: a code running its time loop from a device
   pool reserved at start-up, or one recording its step into its own stream capture.  Bins npoints
   points (coords: device, npoints*dim doubles) into the cells of the uniform mesh of nodes[dim]
   nodes over [O, L], as the context path does: cellid[i] (device, npoints) is the cell or -1 when
   outside; cell_start (device, ncells+1) the exclusive scan of the per-cell counts; order (device,
   npoints, first cell_start[ncells] entries valid) the point indices by cell, input order within a
   cell.  All scratch is a static device array of this library sized for at most
   LAGRBF_NOALLOC_MAX_CELLS cells; larger meshes are rejected with LAGRBF_ERR_ARG_OUTOFRANGE.
   Asynchronous on `stream` (cudaStream_t, NULL = legacy default stream).  The first call on a device
   (that device current) resolves the scratch address, so it should precede any stream capture; the
   address is kept for the life of the process, so the entry point must not be used after
   cudaDeviceReset or from a context other than the device's primary context.
   Calls that overlap on one device share the scratch and race: keep them on one stream. */
#define LAGRBF_NOALLOC_MAX_CELLS (1 << 20)
LAGRBF_EXPORT int lagrbf_gpu_bin_points_noalloc(int32_t dim, const int32_t *nodes, const double *O, const double *L,
                                                int32_t npoints, const double *coords, int32_t *cellid,
                                                int32_t *cell_start, int32_t *order, void *stream);

#ifdef __cplusplus
}
#endif
#endif
