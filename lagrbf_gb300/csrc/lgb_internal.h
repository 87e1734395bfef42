/*
 * lgb_internal.h -- state shared by the C host layer (lgb_host.c) and the CUDA operations
 * (lgb_bin.cu, lgb_eval32_{2,3}d.cu, lgb_eval64.cu, lgb_factor.cu, lgb_step.cu, lgb_noalloc.cu).  Plain C: device memory appears as
 * typed pointers, streams as void*.
 *
 * HBM layout of one context (all arrays device-resident for the lifetime of the dataset):
 *   data swarm      xd[nd*dim] f64 (fill order), fd[nd*F] f64,
 *                   cell_d[nd], cstart[ncells+1], sorted[nd] (fill index of the s-th point in
 *                   cell order), xs[nd*dim] f64 and xr[nd*4] f32 (cell order; xr is relative to
 *                   the point's own cell origin), fs[nd*F] f64 (cell order)
 *   patches         pm[nnodes] sizes, slot[nnodes*8] offset of each adjacent cell inside the
 *                   patch, coff[nnodes+1] i64 pool offsets (points), c64/c32 coefficient pools
 *                   [sum_k m_k * F] laid out [patch][point][field], foff/fac packed lower
 *                   Cholesky factors (only when factors are kept), setup/solved flags
 *   particle swarm  xp[np*dim], fields[np*F], vel[np*dim], x0[np*dim], vadv[7][np*dim] f64,
 *                   cell_p[np], alive[np]; per-stage binning pcount/pstart[ncells+1],
 *                   pfill[ncells], plist[np], chunk_start[ncells+1]
 */
#ifndef LGB_INTERNAL_H
#define LGB_INTERNAL_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum { LGB_KERNEL_LINEAR = 0, LGB_KERNEL_WENDLAND_C0, LGB_KERNEL_WENDLAND_C2, LGB_KERNEL_BUMP,
       LGB_KERNEL_MQ, LGB_KERNEL_IMQ, LGB_KERNEL_GAUSSIAN };
enum { LGB_RK1 = 0, LGB_RK2 = 1, LGB_RK4 = 2, LGB_DOPRI = 3 };
enum { LGB_A_FACTOR = 0, LGB_A_KSP = 1, LGB_A_KSP_ASMB = 2 };
enum { LGB_PREC_FP64 = 0, LGB_PREC_FP32 = 1 };
/* Device-side analytical velocity fields (LAGRBF_VFIELD_* of the public header). */
enum { LGB_VF_NONE = 0, LGB_VF_ROTATION = 1, LGB_VF_CELLULAR = 2, LGB_VF_ABC = 3, LGB_VF_FOURIER = 4 };

/* Largest evaluation work unit (particles of one cell handled by one CTA); the actual capacity
   (d->chunk_cap, a multiple of 64) is chosen from the particles-per-cell histogram. */
#define LGB_CHUNK_MAX 256

/* FP32 record blocks streamed by the evaluation kernel (lgb_evalrec.cuh): per cell, the data
   points of its 3^dim neighbour cells in LGB_NVSEG virtual segments (3D: the centre cell twice,
   with the coefficients of corners 0-3 and of corners 4-7); a record is 2*dim coordinate floats
   and 2 floats per (field, involved patch), padded to 16 bytes. */
#define LGB_NVSEG(dim) ((dim) == 3 ? 28 : 9)
#define LGB_REC2_LEN(dim, ninv, fp) (((2 * (dim) + 2 * (ninv) * (fp) + 3) / 4) * 4)
/* Patch-size classes of the set-up / solve launches: class c holds the patches of up to
   32 * 2^c points (the last class every larger one); LGB_FACT_T is the CTA size of a class without a
   measured entry.  A class with CTAs of T threads keeps 1024 / T of them in flight per SM. */
#define LGB_NCLS 8
#define LGB_FACT_T 128
#ifdef __CUDACC__
#define LGB_HD __host__ __device__
#else
#define LGB_HD
#endif
static inline LGB_HD int lgb_patch_class(int m)
{
  int c = 0;
  while (c < LGB_NCLS - 1 && m > (32 << c)) c++;
  return c;
}
/* FP32 record of one data point as the gather kernel stages it in shared memory: a header {x, x, y,
   y, z, z, 0, 0} (coordinates relative to the evaluating cell's origin, each twice so that one
   64-bit pair holds a coordinate for two particles), then the coefficients of the ninv corner
   patches that contain the point, field-major (field f, patch j at f*ninv + j), each stored
   LGB_REC32_DUP times, padded to a multiple of 16 bytes. */
#define LGB_REC32_HEAD 8
#ifndef LGB_REC32_DUP
#define LGB_REC32_DUP 1
#endif
#define LGB_REC32_LEN(ninv, fp) (((LGB_REC32_HEAD + (ninv) * (fp) * LGB_REC32_DUP + 3) / 4) * 4)

/* PU mesh geometry (DMDA with Q1 elements): nodes are patches, elements are cells. */
typedef struct {
  int dim, nen, kernel;
  int n[3];        /* nodes per axis (1 beyond dim)                      */
  int nc[3];       /* cells per axis (1 beyond dim)                      */
  int nnodes, ncells;
  int wr;          /* weight-support half width in node spacings          */
  double O[3], L[3], h[3];
  double rh[3];    /* 1 / h, for the weight-support node range */
  double eps_w, eps_r;
  double rad_w;    /* 1 / eps_w: the weight support radius as the kernels compute it */
  /* Cell faces as integer keys (lgb_locate): per axis d, bkey[boff[d] + k - 1] is the key of the
     smallest coordinate whose cell index floor((x - O) / h) reaches k (k = 1 .. n[d] - 2), okey /
     lkey the keys of O and L.  Device memory; NULL: locate by the FP64 division. */
  const long long *bkey;
  int boff[3];
  long long okey[3], lkey[3];
} lgb_geom;

/* Device-resident control block of the advection loop: the scalars of
   InternalForwardAdvectionLoop (time_loop.c:39-100) and of the schemes that kernels read. */
typedef struct {
  double t, t_next;
  double dt;           /* step of the current internal step                          */
  double dt_adv;       /* advection context dt (DOPRI stores its adapted step here)   */
  double cfl_fac, cfl_radius;
  double dopri_fac, dopri_fac_min, dopri_fac_max, dopri_atol, dopri_rtol;
  double rmin, rmax;
  double dopri_error;
  unsigned long long n2max_bits;  /* atomicMax target: 1 + bits of the largest |v|^2 of a
                                     live particle (0: none); the CFL step is computed from it */
  unsigned long long maxerr_bits; /* atomicMax target (bits of a non-negative double) */
  int any_alive;
  int scheme;
  int steps;
  int np_alive;
  long long particle_steps;
  double eval_flops;   /* accumulated algorithmic flops of evaluation launches   */
  double eval_bytes;   /* accumulated algorithmic bytes of evaluation launches   */
  int nwork;           /* patches queued for set-up / solve                       */
  int factor_error;    /* first non-positive pivot row (1-based), 0 if none        */
  int factor_node;     /* patch with that pivot                                    */
  int nfactored;
  double factor_flops;
  int nwork_c[LGB_NCLS];  /* queued patches of each size class (the class work lists)      */
  int eval_error;      /* a bounded wait of the evaluation kernel gave up */
  int pp_left;         /* per-particle Dormand-Prince: particles still short of t_next   */
  double dt_cfl_ext;   /* > 0: the CFL step agreed over ranks (replaces the local one)     */
  long long loop_iter; /* internal steps of the current device-side step loop             */
  long long loop_cap;  /* its limit (the loop then stops and the host continues step by step) */
  double pp_hmin;      /* per-particle Dormand-Prince: steps below this are accepted      */
} lgb_ctrl;

typedef struct {
  lgb_geom g;
  int F;               /* n_interpolation_fields */
  int prec;            /* LGB_PREC_*             */
  int solve_method;
  int keep_factors;
  /* data swarm */
  int nd, nd_cap;
  double *xd, *fd, *xs, *fs;
  float *xr;
  int *cell_d, *cstart, *sorted, *dfill, *dtmp;
  int max_cell_pts;
  /* patches */
  int *pm, *slot, *setup, *solved, *work, *status;
  int *need;          /* 2*nnodes ints: flags, also borrowed as nnodes int64 scratch */
  long long *coff, *foff;
  long long coef_cap, fac_cap;
  double *c64, *fac;
  float *c32;
  int max_patch;
  double *ws;          /* factorisation workspace: a pool the class launches share        */
  double *kappa;       /* per-patch 1-norm condition estimates (nnodes), when cond_on    */
  int cond_on;
  /* per-particle adaptive Dormand-Prince (option dopri_per_particle): time reached, next step, step
     of the current sweep, and whether the particle takes part in the sweep */
  int dopri_pp;
  int setup_all;       /* option setup_all_patches: every patch is set up, not only those of cells
                          holding particles */
  double *tp, *hp, *hcur;
  int *active;
  long long ws_stride; /* pool size (doubles) */
  int nws;             /* CTAs of the largest class launch (0: no workspace) */
  /* patch-size classes: work-list region (cls_off, nodes of the class: cls_cap), CTA size, grid
     and workspace slot stride (doubles) of each class launch; cls_off_dev on the device */
  int cls_off[LGB_NCLS + 1], cls_cap[LGB_NCLS], cls_threads[LGB_NCLS], cls_grid[LGB_NCLS];
  long long cls_stride[LGB_NCLS];
  int *cls_off_dev;
  int factor_threads;  /* option factor_threads: one CTA size for every class (0: the table) */
  /* particle swarm */
  int np, np_cap;
  double *xp, *fields, *vel, *x0, *vadv;
  int *cell_p, *alive, *pcount, *pstart, *pfill, *plist, *chunk_start;
  int max_chunks;
  int chunk_cap;       /* particles per evaluation work unit */
  /* precomputed FP32 record blocks streamed by TMA (NULL: gather staging) */
  float *rec32;
  long long *rec_off;
  unsigned char *cdirty; /* [ncells] cells whose record blocks the next rebuild must write */
  long long *bkey_buf; /* device storage of g.bkey (cell-face keys) */
  long long rec_cap;
  int rec_fp;          /* fields per record (= dim) */
  int eval_poll_limit; /* polls of the evaluation kernel's bounded waits (0: the default)     */
  int eval_withhold;   /* test hook: the evaluation kernel arms its staging waits, copies nothing */
  /* scratch for scans */
  int *scan_tmp;
  long long *scan_tmp64;
  /* device-side analytical velocity: kind, parameters (device) and their count */
  int vfield, vfield_np;
  double *vfield_par;
  /* control */
  lgb_ctrl *ctrl;
  int smem_optin;      /* cudaDevAttrMaxSharedMemoryPerBlockOptin */
  int nsm;
} lgb_dev;

/* ---- operations implemented in CUDA (each returns a cudaError_t as int, 0 = success) ---- */
/* lgb_bin.cu */
int lgb_op_locate(const lgb_geom *g, int n, const double *x, int *cell, int *alive, int *counts, int *nbad,
                  void *stream);
int lgb_op_scan_i32(int n, const int *in, int *out, int *tmp, void *stream);
int lgb_op_scan_i64(int n, const long long *in, long long *out, long long *tmp, void *stream);
int lgb_op_scatter(int n, const int *cell, const int *alive, const int *start, int *fill, int *list, void *stream);
int lgb_op_data_arrange(lgb_dev *d, void *stream);      /* xs, xr, fs, patch sizes, slots, offsets */
int lgb_op_data_values(lgb_dev *d, void *stream);       /* fs only (values changed)                */
int lgb_op_bin_particles(lgb_dev *d, int mark_dead, void *stream); /* cell_p, pcount, pstart, plist, chunks */
/* the same, listing for evaluation only the particles with active[p] != 0 (all are located) */
int lgb_op_bin_particles_mask(lgb_dev *d, int mark_dead, const int *active, void *stream);
int lgb_op_mark_patches(lgb_dev *d, void *stream);      /* queue patches touched by live particles */
/* lgb_factor.cu */
int lgb_op_factor(lgb_dev *d, void *stream);            /* set up / solve queued patches */
/* lgb_eval.cu */
int lgb_op_eval(lgb_dev *d, int nf_first, int nf, double *out, int out_stride, void *stream);
int lgb_op_weights(lgb_dev *d, double *w, void *stream);
int lgb_op_build_records(lgb_dev *d, int force, void *stream);
/* lgb_step.cu */
int lgb_op_stage(lgb_dev *d, int scheme, int stage, void *stream);
int lgb_op_dopri_error(lgb_dev *d, void *stream);
int lgb_op_ctrl(lgb_dev *d, int what, void *stream);
enum { LGB_CTRL_BEGIN_STEP = 0, LGB_CTRL_END_STEP = 1, LGB_CTRL_RESET_CFL = 2, LGB_CTRL_DOPRI_DT = 3,
       LGB_CTRL_BEGIN_SWEEP = 4, LGB_CTRL_END_SWEEP = 5 };
/* per-particle Dormand-Prince: tp = t (and hp = dt_adv where unset); the sweep's steps; the error,
   acceptance and next step of every particle in the sweep */
int lgb_op_pp_init(lgb_dev *d, double t, void *stream);
int lgb_op_pp_begin(lgb_dev *d, void *stream);
int lgb_op_pp_accept(lgb_dev *d, void *stream);
int lgb_op_copy_velocity(lgb_dev *d, void *stream);     /* vel <- fields[:, :dim] */
/* Condition of the device-side step loop (a conditional while node of the step graph, handle =
   a cudaGraphConditionalHandle): continue while t < t_next, no error flag is set and the
   iteration limit is not reached. */
int lgb_op_loop_cond(lgb_dev *d, unsigned long long handle, void *stream);
int lgb_op_count_alive(lgb_dev *d, void *stream);
int lgb_op_velocity_field(lgb_dev *d, void *stream);    /* vel <- analytical field at live particles */
int lgb_device_info(int *nsm, int *smem_optin);
/* Output rows by pid (inv: nglobal ints of scratch, bad: one int, set when a pid is out of range);
   coords / fields / pidx may be host pointers the device can access. */
int lgb_op_output_rows(int n, const long long *pid, const int *alive, int nglobal, int *inv, int *bad, int dim,
                       const double *x, double *coords, int nf, const double *src, double *fields, long long *pidx,
                       int nsm, void *stream);
/* Copies `words` 8-byte words from a host array that the device reads directly (pageable memory
   through the GPU's address translation) into device memory; stream-ordered. */
int lgb_op_copy_in(double *dst, const double *src, long long words, int nsm, void *stream);
int lgb_op_check_coords(const lgb_geom *g, int n, const double *x, const double *prev, int *flags, int nsm,
                        void *stream);
/* Sets the calling thread's error message (returned by lagrbf_gpu_last_error); returns code. */
int lgb_set_error_msg(int code, const char *msg);
long long lgb_launch_count(void);

#ifdef __cplusplus
}
#endif
#endif
