/*
 * lgb_host.c -- C host layer of liblagrbf.so: the LagRBF ctypes surface (include/lagrbf.h,
 * section 1), the options store that stands in for PETSc's options database (section 2), and the
 * GPU-level extension (section 3).  Orchestrates the CUDA operations of lgb_*.cu on one stream
 * per context; an internal advection step is captured once as a CUDA graph and replayed.
 *
 * Semantics follow the reference on one MPI rank:
 *   lagrbf_create            -> Interface_LagRBFCreate (src/interface/interface_ctx.c:54-77)
 *   lagrbf_fill_swarm        -> FillDataSwarm / FillInterpSwarm (src/interface/interface_utils.c:68-165)
 *   lagrbf_interpolation     -> LagRBF_PartitionsSetUp + RBFInterpolation("fields")
 *                               (src/interface/interface_interp.c:83-96)
 *   lagrbf_output            -> Interface_Output_Allreduce (src/interface/interface_utils.c:286-339)
 *   lagrbf_reset_coefficients-> LagRBF_PartitionsReset (src/partitions/partition.c:494-524)
 *   lagrbf_advect_interpolate-> InternalForwardAdvectionLoop (src/time_loop.c:39-100)
 *   lagrbf_avect_analytical  -> ForwardAnalyticalAdvection (src/time_loop.c:176-221)
 * Conventions fixed where the reference delegates to PETSc: a point is located in cell
 * floor((x-O)/h) per axis (x == L in the last cell); a particle that leaves [O, L] during
 * advection is removed from the swarm (its output rows are zero); data points keep their fill
 * order inside a cell.  If the data coordinates change while factors are kept (A_FACTOR, A_KSP),
 * every patch is set up again (the reference would reuse factors built for the old points).
 */
#include "lgb_internal.h"
#include "lgb_factor_tune.h"
#include "../../include/lagrbf.h"

#include <cuda_runtime_api.h>
#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdarg.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ======================================================================================= */
/* errors                                                                                   */
/* ======================================================================================= */
static _Thread_local char g_errmsg[512];

static int set_error(int code, const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_errmsg, sizeof(g_errmsg), fmt, ap);
  va_end(ap);
  if (getenv("LAGRBF_VERBOSE")) fprintf(stderr, "lagrbf error %d: %s\n", code, g_errmsg);
  return code;
}

LAGRBF_EXPORT const char *lagrbf_gpu_last_error(void) { return g_errmsg; }

int lgb_set_error_msg(int code, const char *msg) { return set_error(code, "%s", msg); }

/* Mesh dimension and number of interpolation fields of a context (file loaders). */
int lgb_ctx_dims(void *ctx, int *dim, int *nfields);

#define CU(call)                                                                                    \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess)                                                                          \
      return set_error(e_ == cudaErrorMemoryAllocation ? LAGRBF_ERR_MEM : LAGRBF_ERR_GPU, "%s: %s (%s:%d)", \
                       #call, cudaGetErrorString(e_), __FILE__, __LINE__);                          \
  } while (0)
/* CU with a cleanup statement (freeing host buffers) run before the error return */
#define CUF(call, cleanup)                                                                          \
  do {                                                                                              \
    cudaError_t e_ = (call);                                                                        \
    if (e_ != cudaSuccess) {                                                                        \
      cleanup;                                                                                      \
      return set_error(e_ == cudaErrorMemoryAllocation ? LAGRBF_ERR_MEM : LAGRBF_ERR_GPU, "%s: %s (%s:%d)", \
                       #call, cudaGetErrorString(e_), __FILE__, __LINE__);                          \
    }                                                                                               \
  } while (0)
#define OP(call)                                                                                    \
  do {                                                                                              \
    int e_ = (call);                                                                                \
    if (e_) return set_error(LAGRBF_ERR_GPU, "%s: %s (%s:%d)", #call, cudaGetErrorString((cudaError_t)e_), \
                             __FILE__, __LINE__);                                                   \
  } while (0)
#define TRY(call) do { int e_ = (call); if (e_) return e_; } while (0)

/* ======================================================================================= */
/* options store                                                                            */
/* ======================================================================================= */
typedef struct { char *key, *val; } opt_t;
static opt_t *g_opts = NULL;
static int g_nopts = 0, g_capopts = 0;
static pthread_mutex_t g_optlock = PTHREAD_MUTEX_INITIALIZER;

static const char *strip_dash(const char *k) { while (*k == '-') k++; return k; }

LAGRBF_EXPORT int lagrbf_options_set_value(const char *name, const char *value)
{
  int i;
  if (!name) return set_error(LAGRBF_ERR_ARG_NULL, "option name is NULL");
  name = strip_dash(name);
  pthread_mutex_lock(&g_optlock);
  for (i = 0; i < g_nopts; i++)
    if (strcmp(g_opts[i].key, name) == 0) {
      free(g_opts[i].val);
      g_opts[i].val = strdup(value ? value : "");
      pthread_mutex_unlock(&g_optlock);
      return 0;
    }
  if (g_nopts == g_capopts) {
    int cap = g_capopts ? 2 * g_capopts : 32;
    opt_t *no = (opt_t *)realloc(g_opts, sizeof(opt_t) * (size_t)cap);
    if (!no) {
      pthread_mutex_unlock(&g_optlock);
      return set_error(LAGRBF_ERR_MEM, "out of host memory");
    }
    g_opts = no;
    g_capopts = cap;
  }
  g_opts[g_nopts].key = strdup(name);
  g_opts[g_nopts].val = strdup(value ? value : "");
  g_nopts++;
  pthread_mutex_unlock(&g_optlock);
  return 0;
}

LAGRBF_EXPORT int lagrbf_options_clear(void)
{
  int i;
  pthread_mutex_lock(&g_optlock);
  for (i = 0; i < g_nopts; i++) { free(g_opts[i].key); free(g_opts[i].val); }
  g_nopts = 0;
  pthread_mutex_unlock(&g_optlock);
  return 0;
}

LAGRBF_EXPORT int lagrbf_options_get_value(const char *name, char *buf, int32_t buflen)
{
  int i, found = 0;
  if (!name) return 0;
  name = strip_dash(name);
  pthread_mutex_lock(&g_optlock);
  for (i = 0; i < g_nopts; i++)
    if (strcmp(g_opts[i].key, name) == 0) {
      if (buf && buflen > 0) { strncpy(buf, g_opts[i].val, (size_t)buflen - 1); buf[buflen - 1] = 0; }
      found = 1;
      break;
    }
  pthread_mutex_unlock(&g_optlock);
  return found;
}

/* PETSc options-file syntax: whitespace-separated "-key [value]" tokens, '#' starts a comment. */
LAGRBF_EXPORT int lagrbf_options_insert_file(const char *path)
{
  FILE *f;
  char line[4096];
  if (!path) return set_error(LAGRBF_ERR_ARG_NULL, "options file path is NULL");
  f = fopen(path, "r");
  if (!f) return set_error(LAGRBF_ERR_ARG_WRONG, "cannot open options file %s", path);
  while (fgets(line, sizeof(line), f)) {
    char *hash = strchr(line, '#'), *tok, *save = NULL, *key = NULL;
    if (hash) *hash = 0;
    for (tok = strtok_r(line, " \t\r\n", &save); tok; tok = strtok_r(NULL, " \t\r\n", &save)) {
      int is_key = (tok[0] == '-' && !(tok[1] >= '0' && tok[1] <= '9') && tok[1] != '.');
      if (is_key) {
        if (key) lagrbf_options_set_value(key, "true");
        key = tok;
      } else if (key) {
        lagrbf_options_set_value(key, tok);
        key = NULL;
      }
    }
    if (key) lagrbf_options_set_value(key, "true");
  }
  fclose(f);
  return 0;
}

static int opt_str(const char *k, char *buf, int n) { return lagrbf_options_get_value(k, buf, n); }

static int opt_int(const char *k, int *v)
{
  char b[256];
  if (!opt_str(k, b, sizeof(b))) return 0;
  *v = (int)strtol(b, NULL, 10);
  return 1;
}

static int opt_real(const char *k, double *v)
{
  char b[256];
  if (!opt_str(k, b, sizeof(b))) return 0;
  *v = strtod(b, NULL);
  return 1;
}

static int opt_bool(const char *k, int *v)
{
  char b[64];
  if (!opt_str(k, b, sizeof(b))) return 0;
  *v = !(b[0] == '0' || b[0] == 'f' || b[0] == 'F' || b[0] == 'n' || b[0] == 'N');
  return 1;
}

/* Comma (or whitespace) separated arrays, like PetscOptionsGetRealArray. Returns entries read. */
static int opt_real_array(const char *k, double *v, int nmax)
{
  char b[1024], *p, *e;
  int n = 0;
  if (!opt_str(k, b, sizeof(b))) return -1;
  for (p = b; *p && n < nmax;) {
    while (*p == ',' || *p == ' ' || *p == '[' || *p == ']') p++;
    if (!*p) break;
    v[n] = strtod(p, &e);
    if (e == p) break;
    n++;
    p = e;
  }
  return n;
}

static int opt_int_array(const char *k, int *v, int nmax)
{
  double t[16];
  int n = opt_real_array(k, t, nmax < 16 ? nmax : 16), i;
  for (i = 0; i < n; i++) v[i] = (int)t[i];
  return n;
}

/* ======================================================================================= */
/* context                                                                                  */
/* ======================================================================================= */
typedef int (*vfn_t)(double *, double *, void *);
typedef int (*vfnb_t)(int32_t, int32_t, double *, double *, void *);

#define NPROF 16
typedef struct lgb_ctx_s {
  lgb_dev d;
  cudaStream_t stream;
  /* configuration (LagRBFSetFromOptions) */
  int advection, scheme, use_graph, device_loop;
  double dt0, cfl_fac, rmin, rmax;
  double dopri[5];
  /* host mirrors */
  int64_t *pid_d, *pid_p;
  int pid_d_cap, pid_p_cap;
  /* direct output: device copy of the particle pids, pid -> swarm index scratch, status flag */
  int out_direct;        /* option output_direct and the device reads/writes pageable host memory:
                            output rows written and data arrays read by the device directly */
  long long *pidd;
  int pidd_cap, pidd_valid;
  int *out_inv, *out_bad;
  int *chk_flags;  /* flags of the device-side coordinate check of lagrbf_fill_swarm (data) */
  int xd_valid;    /* d->xd holds the coordinates of the last completed data fill, input order */
  long long out_inv_cap;
  double *hx_d;          /* last filled data coordinates (change detection) */
  int data_filled, points_filled;
  vfn_t vfn;
  vfnb_t vfnb;
  void *vuser;
  /* dataset borrowed from another context (lagrbf_gpu_share_dataset): read-only, not freed here */
  struct lgb_ctx_s *shared_from;
  int all_ready;       /* setup_all_patches and every patch set up and solved for the current data */
  /* coupling of sharded runs: element-wise max over the ranks of {-(CFL step), DOPRI error} */
  int (*reduce)(double *, int32_t, void *);
  void *ruser;
  /* graph of one internal step */
  cudaGraphExec_t graph;
  int graph_valid, graph_mode; /* graph_mode: 1 when the captured step is analytical */
  long long graph_launches, graph_eval_launches;
  /* the step inside a device-side while loop: one launch advances a whole advection interval */
  cudaGraphExec_t wgraph;
  int wgraph_valid, wgraph_mode, wgraph_failed;
  long long wgraph_launches, wgraph_eval_launches;
  /* pinned control copy */
  lgb_ctrl *hctrl;
  /* profiling */
  int profiling;
  cudaEvent_t ev[2 * NPROF];
  int nev;
  double eval_ms, factor_ms;
  long long eval_launches, launches_graph;
  long long launch_base;
} lgb_ctx;

static void *dalloc(size_t bytes, int *err)
{
  void *p = NULL;
  if (bytes == 0) bytes = 16;
  if (cudaMalloc(&p, bytes) != cudaSuccess) { *err = 1; return NULL; }
  return p;
}

#define DFREE(p) do { if (p) { cudaFree(p); (p) = NULL; } } while (0)

static void invalidate_graph(lgb_ctx *c)
{
  if (c->graph_valid) cudaGraphExecDestroy(c->graph);
  c->graph_valid = 0;
  if (c->wgraph_valid) cudaGraphExecDestroy(c->wgraph);
  c->wgraph_valid = 0;
}

static void free_data(lgb_dev *d)
{
  DFREE(d->xd); DFREE(d->fd); DFREE(d->xs); DFREE(d->fs); DFREE(d->xr);
  DFREE(d->cell_d); DFREE(d->sorted); DFREE(d->dtmp);
  d->nd_cap = 0;
}

static void free_particles(lgb_dev *d)
{
  DFREE(d->xp); DFREE(d->fields); DFREE(d->vel); DFREE(d->x0); DFREE(d->vadv);
  DFREE(d->cell_p); DFREE(d->alive); DFREE(d->plist);
  DFREE(d->tp); DFREE(d->hp); DFREE(d->hcur); DFREE(d->active);
  d->np_cap = 0;
}

/* The dataset arrays a sharing context borrows (lagrbf_gpu_share_dataset). */
static void borrow_dataset(lgb_dev *d, const lgb_dev *o)
{
  d->xd = o->xd; d->fd = o->fd; d->xs = o->xs; d->fs = o->fs; d->xr = o->xr;
  d->cell_d = o->cell_d; d->cstart = o->cstart; d->sorted = o->sorted;
  d->pm = o->pm; d->slot = o->slot; d->setup = o->setup; d->solved = o->solved;
  d->coff = o->coff; d->foff = o->foff; d->c64 = o->c64; d->c32 = o->c32; d->fac = o->fac;
  d->rec32 = o->rec32; d->rec_off = o->rec_off;
  d->nd = o->nd; d->max_cell_pts = o->max_cell_pts; d->max_patch = o->max_patch;
  d->coef_cap = o->coef_cap; d->fac_cap = o->fac_cap; d->rec_cap = o->rec_cap; d->rec_fp = o->rec_fp;
  d->keep_factors = o->keep_factors;
}

static void unborrow_dataset(lgb_dev *d)
{
  d->xd = d->fd = d->xs = d->fs = NULL;
  d->xr = NULL;
  d->cell_d = d->cstart = d->sorted = NULL;
  d->pm = d->slot = d->setup = d->solved = NULL;
  d->coff = d->foff = NULL;
  d->c64 = d->fac = NULL;
  d->c32 = d->rec32 = NULL;
  d->rec_off = NULL;
  d->nd = 0;
}

static void destroy_ctx(lgb_ctx *c)
{
  lgb_dev *d = &c->d;
  int i;
  if (!c) return;
  if (c->stream) cudaStreamSynchronize(c->stream);
  invalidate_graph(c);
  if (c->shared_from) unborrow_dataset(d);
  free_data(d);
  free_particles(d);
  DFREE(d->cstart); DFREE(d->dfill); DFREE(d->pm); DFREE(d->slot); DFREE(d->setup); DFREE(d->solved);
  DFREE(d->need); DFREE(d->work); DFREE(d->status); DFREE(d->coff); DFREE(d->foff); DFREE(d->c64); DFREE(d->kappa);
  DFREE(d->c32); DFREE(d->fac); DFREE(d->ws); DFREE(d->pcount); DFREE(d->pstart); DFREE(d->pfill);
  DFREE(d->chunk_start); DFREE(d->scan_tmp); DFREE(d->scan_tmp64); DFREE(d->ctrl);
  DFREE(d->rec32); DFREE(d->rec_off); DFREE(d->bkey_buf); DFREE(d->cls_off_dev); DFREE(d->cdirty);
  for (i = 0; i < 2 * NPROF; i++) if (c->ev[i]) cudaEventDestroy(c->ev[i]);
  if (c->hctrl) cudaFreeHost(c->hctrl);
  if (c->stream) cudaStreamDestroy(c->stream);
  DFREE(c->pidd); DFREE(c->out_inv); DFREE(c->out_bad); DFREE(c->chk_flags); DFREE(d->vfield_par);
  free(c->pid_d); free(c->pid_p); free(c->hx_d);
  free(c);
}

/* LagRBFSetFromOptions + PUSetFromOptions + PUCreateDMDA + ComputeSupport/ShapeFactor */
/* The device's order-preserving integer key of a double (lgb_key in lgb_common.cuh). */
static long long face_key(double v)
{
  long long b;
  memcpy(&b, &v, sizeof b);
  if (b == (long long)0x8000000000000000ULL) b = 0;
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

static double key_double(long long k)
{
  double v;
  if (k < 0) k ^= 0x7fffffffffffffffLL;
  memcpy(&v, &k, sizeof v);
  return v;
}

/* Cell faces of the PU mesh as the device's cell location uses them: per axis and k = 1 .. n-2 the
   smallest coordinate x in [O, L] with floor((x - O) / h) >= k.  The predicate is monotone in x,
   so the face is found by bisection over the integer keys of [O, L] (64 steps at most; IEEE
   subtraction, division and floor give the same result here as on the device). */
static int build_face_keys(lgb_dev *d, cudaStream_t stream)
{
  lgb_geom *g = &d->g;
  int dim = g->dim, total = 0, ax, k, err = 0;
  long long *hk;
  for (ax = 0; ax < dim; ax++) total += (g->n[ax] > 2) ? g->n[ax] - 2 : 0;
  for (ax = 0; ax < 3; ax++) {
    g->okey[ax] = face_key(g->O[ax]);
    g->lkey[ax] = face_key(g->L[ax]);
  }
  hk = (long long *)malloc(sizeof(long long) * (size_t)(total > 0 ? total : 1));
  if (!hk) return 0;
  total = 0;
  for (ax = 0; ax < dim; ax++) {
    const double O = g->O[ax], h = g->h[ax];
    g->boff[ax] = total;
    for (k = 1; k <= g->n[ax] - 2; k++) {
      long long lo = g->okey[ax], hi = g->lkey[ax]; /* predicate false at lo (x = O), true at hi */
      if (!(floor((key_double(hi) - O) / h) >= (double)k)) { free(hk); return 0; }
      while ((unsigned long long)hi - (unsigned long long)lo > 1ull) { /* unsigned: no overflow */
        const long long mid = (long long)((unsigned long long)lo + ((unsigned long long)hi - (unsigned long long)lo) / 2);
        if (floor((key_double(mid) - O) / h) >= (double)k) hi = mid;
        else lo = mid;
      }
      hk[total++] = hi;
    }
  }
  d->bkey_buf = (long long *)dalloc(sizeof(long long) * (size_t)(total > 0 ? total : 1), &err);
  if (err) { free(hk); return 0; }
  if (total > 0 && cudaMemcpyAsync(d->bkey_buf, hk, sizeof(long long) * (size_t)total, cudaMemcpyHostToDevice,
                                   stream) != cudaSuccess) {
    free(hk);
    return 0;
  }
  cudaStreamSynchronize(stream);
  free(hk);
  g->bkey = d->bkey_buf;
  return 0;
}

static int read_options(lgb_ctx *c)
{
  lgb_dev *d = &c->d;
  lgb_geom *g = &d->g;
  int dim = 0, n[3] = {0, 0, 0}, nn, k, i;
  double O[3] = {0, 0, 0}, L[3] = {1, 1, 1}, overlap = 1.0, shape = 1.0, box = 0.0, radius;
  char buf[64];
  memset(g, 0, sizeof(*g));
  if (!opt_int("pu_mesh_dim", &dim)) return set_error(LAGRBF_ERR_ARG_WRONG, "option -pu_mesh_dim not provided");
  if (dim != 2 && dim != 3) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "pu_mesh_dim must be 2 or 3, found %d", dim);
  nn = opt_int_array("pu_mesh_n", n, 3);
  if (nn < 0) return set_error(LAGRBF_ERR_ARG_WRONG, "option -pu_mesh_n not provided");
  if (nn != dim) return set_error(LAGRBF_ERR_ARG_SIZ, "option -pu_mesh_n: expected %d entries, found %d", dim, nn);
  nn = opt_real_array("pu_mesh_O", O, 3);
  if (nn >= 0 && nn != dim) return set_error(LAGRBF_ERR_ARG_SIZ, "option -pu_mesh_O: expected %d entries", dim);
  nn = opt_real_array("pu_mesh_L", L, 3);
  if (nn >= 0 && nn != dim) return set_error(LAGRBF_ERR_ARG_SIZ, "option -pu_mesh_L: expected %d entries", dim);
  opt_real("pu_mesh_overlap", &overlap);
  opt_real("pu_mesh_shape_factor", &shape);
  if (!(shape > 0.0)) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "shape factor must be positive, found %g", shape);
  g->dim = dim;
  g->nen = 1 << dim;
  g->nnodes = 1;
  g->ncells = 1;
  for (i = 0; i < 3; i++) {
    if (i < dim) {
      if (n[i] < 2) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "pu_mesh_n[%d] must be >= 2", i);
      if (!(L[i] > O[i])) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "pu_mesh_L must exceed pu_mesh_O");
      g->n[i] = n[i];
      g->nc[i] = n[i] - 1;
      g->O[i] = O[i];
      g->L[i] = L[i];
      g->h[i] = (L[i] - O[i]) / (double)(n[i] - 1);
      g->nnodes *= n[i];
      g->ncells *= n[i] - 1;
      box = (box < L[i] - O[i]) ? L[i] - O[i] : box;
    } else {
      g->n[i] = 1; g->nc[i] = 1; g->O[i] = 0; g->L[i] = 0; g->h[i] = 1.0;
    }
  }
  radius = overlap * box / pow((double)g->nnodes, 1.0 / dim); /* partition_of_unity.c:340-344 */
  g->eps_w = 1.0 / radius;
  g->eps_r = shape * g->eps_w;
  g->rad_w = 1.0 / g->eps_w;
  for (i = 0; i < 3; i++) g->rh[i] = 1.0 / g->h[i];
  g->wr = 1;
  for (i = 0; i < dim; i++) {
    int w = (int)ceil(radius / g->h[i]);
    if (w > g->wr) g->wr = w;
  }
  /* LagRBFSetFromOptions (lagrangian_rbf.c:135-195); C defaults of LagRBFCtxCreate */
  g->kernel = LGB_KERNEL_LINEAR;
  if (opt_int("kernel_type", &k)) g->kernel = k;
  if (g->kernel < 0 || g->kernel > 6) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "unknown kernel type %d", g->kernel);
  d->solve_method = LGB_A_FACTOR;
  if (opt_int("solve_method", &k)) d->solve_method = k;
  if (d->solve_method < 0 || d->solve_method > 2) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "unknown solve method %d", k);
  d->keep_factors = (d->solve_method != LGB_A_KSP_ASMB);
  d->F = 0;
  opt_int("n_interpolation_fields", &d->F);
  if (d->F < 0) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "n_interpolation_fields must be >= 0");
  c->rmin = 0.0;
  c->rmax = DBL_MAX;
  c->cfl_fac = 0.4;
  opt_real("rmin", &c->rmin);
  opt_real("rmax", &c->rmax);
  opt_real("cfl_fac", &c->cfl_fac);
  c->advection = 0;
  opt_bool("advection", &c->advection);
  c->scheme = LGB_DOPRI;
  c->dt0 = 1e-10;
  if (c->advection) {
    opt_int("advection_scheme", &c->scheme);
    if (c->scheme < 0 || c->scheme > 3) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "unknown advection scheme %d", c->scheme);
    opt_real("dt", &c->dt0);
    if (opt_str("velocity_name", buf, sizeof(buf)) && strcmp(buf, "velocity") != 0)
      return set_error(LAGRBF_ERR_SUP, "velocity_name other than \"velocity\" is not supported");
  }
  c->dopri[0] = 0.9; c->dopri[1] = 1.0e-2; c->dopri[2] = 1.0e2; c->dopri[3] = 1.0e-3; c->dopri[4] = 1.0e-3;
  opt_real("dopri_dt_fac", &c->dopri[0]);
  opt_real("dopri_dt_fac_min", &c->dopri[1]);
  opt_real("dopri_dt_fac_max", &c->dopri[2]);
  opt_real("dopri_atol", &c->dopri[3]);
  opt_real("dopri_rtol", &c->dopri[4]);
  d->dopri_pp = 0;
  opt_bool("dopri_per_particle", &d->dopri_pp);
  d->setup_all = 0;
  opt_bool("setup_all_patches", &d->setup_all);
  d->factor_threads = 0;
  if (opt_int("factor_threads", &d->factor_threads) &&
      !(d->factor_threads == 32 || d->factor_threads == 64 || d->factor_threads == 128 || d->factor_threads == 256))
    return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "factor_threads must be 32, 64, 128 or 256");
  d->prec = LGB_PREC_FP64;
  if (opt_str("eval_precision", buf, sizeof(buf))) {
    if (strcmp(buf, "fp32") == 0) d->prec = LGB_PREC_FP32;
    else if (strcmp(buf, "fp64") != 0) return set_error(LAGRBF_ERR_SUP, "eval_precision must be fp32 or fp64");
  }
  c->use_graph = 1;
  opt_bool("use_cuda_graph", &c->use_graph);
  c->device_loop = 1;
  opt_bool("device_loop", &c->device_loop);
  c->out_direct = 1;
  opt_bool("output_direct", &c->out_direct);
  return 0;
}

static int create_ctx(lgb_ctx **out)
{
  lgb_ctx *c = (lgb_ctx *)calloc(1, sizeof(lgb_ctx));
  lgb_dev *d;
  int err = 0, i, nn, nc;
  if (!c) return set_error(LAGRBF_ERR_MEM, "out of host memory");
  d = &c->d;
  if ((i = read_options(c))) { free(c); return i; }
  {
    int dev = -1;
    if (opt_int("cuda_device", &dev) && dev >= 0 && cudaSetDevice(dev) != cudaSuccess) {
      free(c);
      return set_error(LAGRBF_ERR_GPU, "cudaSetDevice(%d) failed", dev);
    }
  }
  if (lgb_device_info(&d->nsm, &d->smem_optin)) { free(c); return set_error(LAGRBF_ERR_GPU, "no CUDA device"); }
  {
    /* direct output needs coherent device access to pageable host memory (host page tables) */
    int dev = 0, pageable = 0, host_pt = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&pageable, cudaDevAttrPageableMemoryAccess, dev);
    cudaDeviceGetAttribute(&host_pt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev);
    c->out_direct = c->out_direct && pageable && host_pt;
  }
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    free(c);
    return set_error(LAGRBF_ERR_GPU, "cudaStreamCreate failed");
  }
  nn = d->g.nnodes;
  nc = d->g.ncells;
  d->cstart = (int *)dalloc(sizeof(int) * (size_t)(nc + 1), &err);
  d->dfill = (int *)dalloc(sizeof(int) * (size_t)nc, &err);
  d->pm = (int *)dalloc(sizeof(int) * (size_t)nn, &err);
  d->slot = (int *)dalloc(sizeof(int) * 8 * (size_t)nn, &err);
  d->setup = (int *)dalloc(sizeof(int) * (size_t)nn, &err);
  d->solved = (int *)dalloc(sizeof(int) * (size_t)nn, &err);
  d->need = (int *)dalloc(sizeof(int) * 2 * (size_t)nn, &err);
  d->work = (int *)dalloc(sizeof(int) * (size_t)nn, &err);
  d->status = (int *)dalloc(sizeof(int) * (size_t)nn, &err);
  d->coff = (long long *)dalloc(sizeof(long long) * (size_t)(nn + 1), &err);
  d->foff = (long long *)dalloc(sizeof(long long) * (size_t)(nn + 1), &err);
  d->pcount = (int *)dalloc(sizeof(int) * (size_t)(nc + 1), &err);
  d->pstart = (int *)dalloc(sizeof(int) * (size_t)(nc + 1), &err);
  d->pfill = (int *)dalloc(sizeof(int) * (size_t)(nc + 1), &err);
  d->chunk_start = (int *)dalloc(sizeof(int) * (size_t)(nc + 1), &err);
  d->cdirty = (unsigned char *)dalloc((size_t)nc, &err);
  d->scan_tmp = (int *)dalloc(sizeof(int) * 4096, &err);
  d->scan_tmp64 = (long long *)dalloc(sizeof(long long) * 4096, &err);
  d->ctrl = (lgb_ctrl *)dalloc(sizeof(lgb_ctrl), &err);
  if (err) { destroy_ctx(c); return set_error(LAGRBF_ERR_MEM, "device allocation failed in lagrbf_create"); }
  if (cudaMallocHost((void **)&c->hctrl, sizeof(lgb_ctrl)) != cudaSuccess) {
    destroy_ctx(c);
    return set_error(LAGRBF_ERR_MEM, "pinned allocation failed");
  }
  if (nc + 1 > 4096 * 2048 || nn + 1 > 4096 * 2048) {
    destroy_ctx(c);
    return set_error(LAGRBF_ERR_SUP, "PU mesh too large (ncells, nnodes <= 8M)");
  }
  build_face_keys(d, c->stream);
  cudaMemsetAsync(d->setup, 0, sizeof(int) * (size_t)nn, c->stream);
  cudaMemsetAsync(d->solved, 0, sizeof(int) * (size_t)nn, c->stream);
  cudaMemsetAsync(d->need, 0, sizeof(int) * 2 * (size_t)nn, c->stream);
  cudaMemsetAsync(d->cstart, 0, sizeof(int) * (size_t)(nc + 1), c->stream);
  cudaMemsetAsync(d->pstart, 0, sizeof(int) * (size_t)(nc + 1), c->stream);
  cudaMemsetAsync(d->chunk_start, 0, sizeof(int) * (size_t)(nc + 1), c->stream);
  cudaMemsetAsync(d->cdirty, 0, (size_t)nc, c->stream);
  memset(c->hctrl, 0, sizeof(lgb_ctrl));
  c->hctrl->dt_adv = c->dt0;
  c->hctrl->cfl_fac = c->cfl_fac;
  c->hctrl->cfl_radius = 1.0 / d->g.eps_w;
  c->hctrl->dopri_fac = c->dopri[0];
  c->hctrl->dopri_fac_min = c->dopri[1];
  c->hctrl->dopri_fac_max = c->dopri[2];
  c->hctrl->dopri_atol = c->dopri[3];
  c->hctrl->dopri_rtol = c->dopri[4];
  c->hctrl->dopri_error = DBL_MAX;
  c->hctrl->rmin = c->rmin;
  c->hctrl->rmax = c->rmax;
  c->hctrl->scheme = c->scheme;
  if (cudaMemcpyAsync(d->ctrl, c->hctrl, sizeof(lgb_ctrl), cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess) {
    destroy_ctx(c);
    return set_error(LAGRBF_ERR_GPU, "initialising the device context failed");
  }
  for (i = 0; i < 2 * NPROF; i++) cudaEventCreate(&c->ev[i]);
  c->launch_base = lgb_launch_count();
  d->chunk_cap = LGB_CHUNK_MAX;
  *out = c;
  return 0;
}

/* ---------------------------------------------------------------------------------------- */
/* swarm filling                                                                            */
/* ---------------------------------------------------------------------------------------- */
/* DMSwarmAssignRankFromDMDA (swarm_utils.c:854-871) on one rank: every coordinate inside [O, L].
   One branch-free pass (vectorised) that also compares the words with `prev` when given: *same = 1
   when all n*dim words are equal.  The first offending point is searched only when one exists. */
static int check_box(const lgb_geom *g, int n, const double *x, const double *prev, int *same)
{
  const int dim = g->dim;
  const double lx = g->O[0], hx = g->L[0], ly = g->O[1], hy = g->L[1];
  const double lz = g->O[dim - 1], hz = g->L[dim - 1];
  uint64_t diff = 0;
  int out = 0, p, d;
  if (dim == 3) {
    for (p = 0; p < n; p++) {
      const double a = x[3 * (size_t)p], b = x[3 * (size_t)p + 1], c = x[3 * (size_t)p + 2];
      out |= (a < lx) | (a > hx) | (b < ly) | (b > hy) | (c < lz) | (c > hz);
    }
  } else {
    for (p = 0; p < n; p++) {
      const double a = x[(size_t)dim * p], b = x[(size_t)dim * p + 1];
      out |= (a < lx) | (a > hx) | (b < ly) | (b > hy);
    }
  }
  if (out) {
    for (p = 0; p < n; p++)
      for (d = 0; d < dim; d++) {
        double v = x[(size_t)p * dim + d];
        if (v < g->O[d] || v > g->L[d])
          return set_error(LAGRBF_ERR_ARG_WRONG, "point %d does not belong to the PU mesh bounding box", p);
      }
  }
  if (same) {
    *same = 0;
    if (prev) {
      const size_t nw = (size_t)n * dim;
      size_t i;
      for (i = 0; i < nw; i++) {
        uint64_t a, b;
        memcpy(&a, &x[i], sizeof a);
        memcpy(&b, &prev[i], sizeof b);
        diff |= a ^ b;
      }
      *same = (diff == 0);
    }
  }
  return 0;
}

/* SwarmFieldAssignUniqueIndex (swarm_utils.c:37-73) on one rank: the resized swarm keeps the first
   min(old, new) pids and zero beyond; new pids are max + 1 + p. */
static void assign_pids(int64_t *pid, int old_n, int new_n)
{
  int64_t mx = 0;
  int p;
  for (p = 0; p < new_n; p++) {
    int64_t v = (p < old_n) ? pid[p] : 0;
    if (v > mx) mx = v;
  }
  for (p = 0; p < new_n; p++) pid[p] = mx + 1 + p;
}

static int grow_pids(int64_t **a, int *cap, int old_n, int n)
{
  if (n > *cap) {
    int64_t *b = (int64_t *)realloc(*a, sizeof(int64_t) * (size_t)n);
    if (!b) return set_error(LAGRBF_ERR_MEM, "out of host memory");
    *a = b;
    *cap = n;
  }
  if (n > old_n) memset(*a + old_n, 0, sizeof(int64_t) * (size_t)(n - old_n));
  return 0;
}

/* Patch-size classes of the set-up / solve launches: per class the work-list region (by the number
   of its patches), the CTA size (option factor_threads, else the measured table), the workspace
   slot of its largest patch (m^2 + m (dim + F) + 17 m + 32 doubles: matrix, coordinates,
   right-hand sides, Cholesky panel rows) and a grid of 1024 / T CTAs per SM; the pool holds the
   largest class grid x slot, at most LGB_FACT_WS_BYTES (a class with bigger slots runs fewer CTAs). */
#define LGB_FACT_WS_BYTES (4LL << 30)
static int plan_classes(lgb_ctx *c)
{
  lgb_dev *d = &c->d;
  int nn = d->g.nnodes, i, k, err = 0, cls_m[LGB_NCLS];
  int *pm = (int *)malloc(sizeof(int) * (size_t)nn);
  long long pool = 0;
  if (!pm) return set_error(LAGRBF_ERR_MEM, "out of host memory");
  CUF(cudaMemcpy(pm, d->pm, sizeof(int) * (size_t)nn, cudaMemcpyDeviceToHost), free(pm));
  for (k = 0; k < LGB_NCLS; k++) { d->cls_cap[k] = 0; cls_m[k] = 0; }
  for (i = 0; i < nn; i++) {
    k = lgb_patch_class(pm[i]);
    d->cls_cap[k]++;
    if (pm[i] > cls_m[k]) cls_m[k] = pm[i];
  }
  free(pm);
  d->cls_off[0] = 0;
  d->nws = 0;
  for (k = 0; k < LGB_NCLS; k++) {
    const long long m = cls_m[k] > 0 ? cls_m[k] : 1;
    const int T = d->factor_threads ? d->factor_threads : lgb_factor_threads[k];
    long long grid = (long long)(1024 / T) * d->nsm;
    d->cls_off[k + 1] = d->cls_off[k] + d->cls_cap[k];
    d->cls_threads[k] = T;
    d->cls_stride[k] = m * m + m * (d->g.dim + d->F) + m * 17 + 32;
    if (grid > d->cls_cap[k]) grid = d->cls_cap[k];
    if (grid * d->cls_stride[k] * 8 > LGB_FACT_WS_BYTES) grid = LGB_FACT_WS_BYTES / (d->cls_stride[k] * 8);
    if (grid < 1 && d->cls_cap[k] > 0) grid = 1;
    d->cls_grid[k] = (int)grid;
    if (grid * d->cls_stride[k] > pool) pool = grid * d->cls_stride[k];
    if (grid > d->nws) d->nws = (int)grid;
  }
  if (!d->cls_off_dev) d->cls_off_dev = (int *)dalloc(sizeof(int) * (LGB_NCLS + 1), &err);
  if (err) return set_error(LAGRBF_ERR_MEM, "class table allocation failed");
  CU(cudaMemcpy(d->cls_off_dev, d->cls_off, sizeof(int) * (LGB_NCLS + 1), cudaMemcpyHostToDevice));
  if (pool > d->ws_stride) {
    DFREE(d->ws);
    d->ws = (double *)dalloc(sizeof(double) * (size_t)(pool > 0 ? pool : 1), &err);
    d->ws_stride = err ? 0 : pool;
    if (err) { d->nws = 0; return set_error(LAGRBF_ERR_MEM, "factorisation workspace allocation failed"); }
  }
  return 0;
}

static int ensure_pools(lgb_ctx *c)
{
  lgb_dev *d = &c->d;
  long long total = 0, ftotal = 0;
  int err = 0, nn = d->g.nnodes;
  CU(cudaMemcpyAsync(&total, d->coff + nn, sizeof(long long), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  if (total * (d->F > 0 ? d->F : 1) > d->coef_cap) {
    DFREE(d->c64); DFREE(d->c32);
    d->coef_cap = total * (d->F > 0 ? d->F : 1);
    d->c64 = (double *)dalloc(sizeof(double) * (size_t)d->coef_cap, &err);
    d->c32 = (float *)dalloc(sizeof(float) * (size_t)d->coef_cap, &err);
    if (err) { d->coef_cap = 0; return set_error(LAGRBF_ERR_MEM, "coefficient pool allocation failed"); }
  }
  if (d->keep_factors) {
    /* packed factor offsets: exclusive scan of m(m+1)/2, computed on the host from pm */
    int *pm = (int *)malloc(sizeof(int) * (size_t)nn), i;
    long long *fo = (long long *)malloc(sizeof(long long) * (size_t)(nn + 1));
    if (!pm || !fo) { free(pm); free(fo); return set_error(LAGRBF_ERR_MEM, "out of host memory"); }
    CUF(cudaMemcpy(pm, d->pm, sizeof(int) * (size_t)nn, cudaMemcpyDeviceToHost), (free(pm), free(fo)));
    for (i = 0; i < nn; i++) { fo[i] = ftotal; ftotal += (long long)pm[i] * (pm[i] + 1) / 2; }
    fo[nn] = ftotal;
    CUF(cudaMemcpy(d->foff, fo, sizeof(long long) * (size_t)(nn + 1), cudaMemcpyHostToDevice), (free(pm), free(fo)));
    free(pm); free(fo);
    if (ftotal > d->fac_cap) {
      DFREE(d->fac);
      d->fac_cap = ftotal;
      d->fac = (double *)dalloc(sizeof(double) * (size_t)ftotal, &err);
      if (err) { d->fac_cap = 0; return set_error(LAGRBF_ERR_MEM, "factor pool allocation failed (%lld doubles)", ftotal); }
    }
  }
  TRY(plan_classes(c));
  return 0;
}

/* Offsets of the precomputed FP32 record blocks (one per cell, neighbour-offset order, dim fields per
   corner patch) and their allocation; disabled (gather staging) when F < dim or when the blocks would
   exceed LAGRBF_RECORDS_MAX_GB (default 16 GB). */
static int ensure_records(lgb_ctx *c)
{
  lgb_dev *d = &c->d;
  const lgb_geom *g = &d->g;
  int nc = g->ncells, cell, vs, err = 0;
  int nvs = LGB_NVSEG(g->dim);
  int *cs;
  long long *off, total = 0, maxbytes = 16LL << 30;
  const char *env = getenv("LAGRBF_RECORDS_MAX_GB");
  if (env) maxbytes = (long long)(atof(env) * (double)(1LL << 30));
  d->rec_fp = g->dim;
  if (d->F < g->dim || maxbytes <= 0) { DFREE(d->rec32); d->rec_cap = 0; return 0; }
  cs = (int *)malloc(sizeof(int) * (size_t)(nc + 1));
  off = (long long *)malloc(sizeof(long long) * (size_t)(nc + 1));
  if (!cs || !off) { free(cs); free(off); return set_error(LAGRBF_ERR_MEM, "out of host memory"); }
  CUF(cudaMemcpy(cs, d->cstart, sizeof(int) * (size_t)(nc + 1), cudaMemcpyDeviceToHost), (free(cs), free(off)));
  for (cell = 0; cell < nc; cell++) {
    int cxy = g->nc[0] * g->nc[1], l = cell / cxy, r = cell - l * cxy, j = r / g->nc[0], i = r - j * g->nc[0];
    off[cell] = total;
    for (vs = 0; vs < nvs; vs++) {
      /* virtual segment vs: neighbour offset o; in 3D the centre cell (o = 13) appears twice, with
         the coefficients of four corner patches each */
      int o = (g->dim == 3 && vs > 13) ? vs - 1 : vs;
      int a = o % 3 - 1, b = (o / 3) % 3 - 1, e = (g->dim == 3) ? o / 9 - 1 : 0;
      int ni = i + a, nj = j + b, nl = l + e, nb, ninv, S;
      if (ni < 0 || ni >= g->nc[0] || nj < 0 || nj >= g->nc[1] || nl < 0 || nl >= g->nc[2]) continue;
      nb = ni + nj * g->nc[0] + nl * cxy;
      ninv = (a == 0 ? 2 : 1) * (b == 0 ? 2 : 1) * ((g->dim == 3 && e == 0) ? 2 : 1);
      if (ninv > 4) ninv = 4;
      S = LGB_REC2_LEN(g->dim, ninv, g->dim);
      total += (long long)(cs[nb + 1] - cs[nb]) * S;
    }
  }
  off[nc] = total;
  free(cs);
  if (total * 4 > maxbytes) {
    free(off);
    DFREE(d->rec32);
    d->rec_cap = 0;
    return 0;
  }
  if (!d->rec_off) d->rec_off = (long long *)dalloc(sizeof(long long) * (size_t)(nc + 1), &err);
  if (total > d->rec_cap) {
    DFREE(d->rec32);
    d->rec32 = (float *)dalloc(sizeof(float) * (size_t)(total > 0 ? total : 4), &err);
    d->rec_cap = err ? 0 : total;
  }
  if (err) { free(off); DFREE(d->rec32); d->rec_cap = 0; return 0; /* fall back to gather staging */ }
  CUF(cudaMemcpy(d->rec_off, off, sizeof(long long) * (size_t)(nc + 1), cudaMemcpyHostToDevice), free(off));
  free(off);
  return 0;
}

static int fill_data(lgb_ctx *c, int n, const double *coords, const double *values, const int64_t *pidx)
{
  lgb_dev *d = &c->d;
  int dim = d->g.dim, F = d->F, err = 0, same_coords;
  int old = d->nd;
  const int prev_ok = c->xd_valid && n == old && n > 0;
  if (c->shared_from)
    return set_error(LAGRBF_ERR_ARG_WRONGSTATE, "the data swarm is shared from another context (read-only)");
  c->all_ready = 0;
  c->xd_valid = 0;
  if (c->out_direct && n > 0) {
    /* the device reads the caller's array: one pass checks the bounding box and compares the words
       with the coordinates already on the device (the host pass below only names an offender) */
    int fl[2] = {0, 0};
    if (!c->chk_flags) c->chk_flags = (int *)dalloc(2 * sizeof(int), &err);
    if (err) return set_error(LAGRBF_ERR_MEM, "coordinate check flags allocation failed");
    OP(lgb_op_check_coords(&d->g, n, coords, prev_ok ? d->xd : NULL, c->chk_flags, d->nsm, c->stream));
    CU(cudaMemcpyAsync(fl, c->chk_flags, sizeof fl, cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    if (fl[0]) TRY(check_box(&d->g, n, coords, NULL, NULL));
    same_coords = prev_ok && !fl[1];
  } else {
    TRY(check_box(&d->g, n, coords, (prev_ok && c->hx_d) ? c->hx_d : NULL, &same_coords));
  }
  TRY(grow_pids(&c->pid_d, &c->pid_d_cap, old, n));
  if (pidx) memcpy(c->pid_d, pidx, sizeof(int64_t) * (size_t)n);
  else assign_pids(c->pid_d, old, n);
  if (n > d->nd_cap) {
    free_data(d);
    d->xd = (double *)dalloc(sizeof(double) * (size_t)n * dim, &err);
    d->fd = (double *)dalloc(sizeof(double) * (size_t)n * (F ? F : 1), &err);
    d->xs = (double *)dalloc(sizeof(double) * (size_t)n * dim, &err);
    d->fs = (double *)dalloc(sizeof(double) * (size_t)n * (F ? F : 1), &err);
    d->xr = (float *)dalloc(sizeof(float) * 4 * (size_t)n, &err);
    d->cell_d = (int *)dalloc(sizeof(int) * (size_t)n, &err);
    d->sorted = (int *)dalloc(sizeof(int) * (size_t)n, &err);
    d->dtmp = (int *)dalloc(sizeof(int) * (size_t)n, &err);
    if (err) return set_error(LAGRBF_ERR_MEM, "data swarm allocation failed (%d points)", n);
    d->nd_cap = n;
    invalidate_graph(c);
  }
  if (n > old && F > 0) CU(cudaMemsetAsync(d->fd + (size_t)old * F, 0, sizeof(double) * (size_t)(n - old) * F, c->stream));
  d->nd = n;
  /* unchanged coordinates (compared word for word above) are already on the device; where the
     device reads pageable host memory it copies the caller's arrays itself */
  if (n > 0 && !same_coords) {
    if (c->out_direct) OP(lgb_op_copy_in(d->xd, coords, (long long)n * dim, d->nsm, c->stream));
    else CU(cudaMemcpyAsync(d->xd, coords, sizeof(double) * (size_t)n * dim, cudaMemcpyHostToDevice, c->stream));
  }
  if (values && n > 0 && F > 0) {
    if (c->out_direct) OP(lgb_op_copy_in(d->fd, values, (long long)n * F, d->nsm, c->stream));
    else CU(cudaMemcpyAsync(d->fd, values, sizeof(double) * (size_t)n * F, cudaMemcpyHostToDevice, c->stream));
  }
  if (same_coords) {
    OP(lgb_op_data_values(d, c->stream));
  } else {
    OP(lgb_op_data_arrange(d, c->stream));
    TRY(ensure_pools(c));
    TRY(ensure_records(c));
    /* membership changed: every patch must be set up again, and every cell's record block is
       rewritten now (no patch set up: zero coefficients), so that cells whose patches stay
       untouched hold no records of the previous data */
    CU(cudaMemsetAsync(d->setup, 0, sizeof(int) * (size_t)d->g.nnodes, c->stream));
    CU(cudaMemsetAsync(d->solved, 0, sizeof(int) * (size_t)d->g.nnodes, c->stream));
    OP(lgb_op_build_records(d, 1, c->stream));
    free(c->hx_d);
    c->hx_d = NULL;
    if (!c->out_direct) { /* host copy for the next comparison (the device compares with d->xd) */
      c->hx_d = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * dim);
      if (n > 0 && c->hx_d) memcpy(c->hx_d, coords, sizeof(double) * (size_t)n * dim);
    }
    invalidate_graph(c);
  }
  CU(cudaStreamSynchronize(c->stream));
  c->data_filled = 1;
  c->xd_valid = 1;
  return 0;
}

/* Work-unit capacity of the evaluation kernel from the particles-per-cell histogram: the cost of a
   capacity C = 64m (m = 1..4, R = 2 particles per thread) is, per work unit, one warp-equivalent of
   block staging plus its active warps plus a third of a warp for each warp left without particles
   (it still stages and occupies the SM). */
static int choose_chunk(lgb_ctx *c)
{
  lgb_dev *d = &c->d;
  int nc = d->g.ncells, i, m, best = 4;
  double bestcost = -1.0;
  int *cnt = (int *)malloc(sizeof(int) * (size_t)(nc + 1));
  if (!cnt) return set_error(LAGRBF_ERR_MEM, "out of host memory");
  CUF(cudaMemcpyAsync(cnt, d->pstart, sizeof(int) * (size_t)(nc + 1), cudaMemcpyDeviceToHost, c->stream), free(cnt));
  CUF(cudaStreamSynchronize(c->stream), free(cnt));
  for (m = 4; m >= 1; m--) {
    double cost = 0.0;
    int cap = 64 * m, twarps = 2 * m;
    for (i = 0; i < nc; i++) {
      int n = cnt[i + 1] - cnt[i], nch, per, aw;
      if (n <= 0) continue;
      nch = (n + cap - 1) / cap;
      per = (n + nch - 1) / nch;
      aw = ((per + 1) / 2 + 31) / 32;
      cost += nch * (1.0 + aw + (twarps - aw) / 3.0);
    }
    if (bestcost < 0.0 || cost < bestcost * 0.98) { bestcost = cost; best = m; }
  }
  free(cnt);
  {
    const char *env = getenv("LAGRBF_CHUNK");
    if (env && atoi(env) >= 64 && atoi(env) <= LGB_CHUNK_MAX) best = atoi(env) / 64;
  }
  if (64 * best != d->chunk_cap) {
    d->chunk_cap = 64 * best;
    invalidate_graph(c);
    OP(lgb_op_bin_particles(d, 0, c->stream)); /* chunk offsets for the new capacity */
  }
  d->max_chunks = d->g.ncells + (d->np + d->chunk_cap - 1) / d->chunk_cap + 1;
  return 0;
}

static int fill_points(lgb_ctx *c, int n, const double *coords, const double *values, const int64_t *pidx)
{
  lgb_dev *d = &c->d;
  int dim = d->g.dim, F = d->F, err = 0, old = d->np;
  TRY(check_box(&d->g, n, coords, NULL, NULL));
  TRY(grow_pids(&c->pid_p, &c->pid_p_cap, old, n));
  if (pidx) memcpy(c->pid_p, pidx, sizeof(int64_t) * (size_t)n);
  else assign_pids(c->pid_p, old, n);
  c->pidd_valid = 0;
  if (n > d->np_cap) {
    /* keep the old field contents of the first `old` particles (the swarm keeps them) */
    double *of = d->fields, *ov = d->vel;
    d->fields = NULL; d->vel = NULL;
    free_particles(d);
    d->xp = (double *)dalloc(sizeof(double) * (size_t)n * dim, &err);
    d->fields = (double *)dalloc(sizeof(double) * (size_t)n * (F ? F : 1), &err);
    d->vel = (double *)dalloc(sizeof(double) * (size_t)n * dim, &err);
    d->x0 = (double *)dalloc(sizeof(double) * (size_t)n * dim, &err);
    d->vadv = (double *)dalloc(sizeof(double) * 7 * (size_t)n * dim, &err);
    d->cell_p = (int *)dalloc(sizeof(int) * (size_t)n, &err);
    d->alive = (int *)dalloc(sizeof(int) * (size_t)n, &err);
    d->plist = (int *)dalloc(sizeof(int) * (size_t)n, &err);
    if (d->dopri_pp) {
      d->tp = (double *)dalloc(sizeof(double) * (size_t)n, &err);
      d->hp = (double *)dalloc(sizeof(double) * (size_t)n, &err);
      d->hcur = (double *)dalloc(sizeof(double) * 2 * (size_t)n, &err);
      d->active = (int *)dalloc(sizeof(int) * (size_t)n, &err);
    }
    if (err) { DFREE(of); DFREE(ov); return set_error(LAGRBF_ERR_MEM, "particle swarm allocation failed (%d points)", n); }
    CU(cudaMemsetAsync(d->fields, 0, sizeof(double) * (size_t)n * (F ? F : 1), c->stream));
    CU(cudaMemsetAsync(d->vel, 0, sizeof(double) * (size_t)n * dim, c->stream));
    if (of && old > 0 && F > 0) CU(cudaMemcpyAsync(d->fields, of, sizeof(double) * (size_t)old * F, cudaMemcpyDeviceToDevice, c->stream));
    if (ov && old > 0) CU(cudaMemcpyAsync(d->vel, ov, sizeof(double) * (size_t)old * dim, cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    DFREE(of); DFREE(ov);
    d->np_cap = n;
    invalidate_graph(c);
  } else if (n > old) {
    if (F > 0) CU(cudaMemsetAsync(d->fields + (size_t)old * F, 0, sizeof(double) * (size_t)(n - old) * F, c->stream));
    CU(cudaMemsetAsync(d->vel + (size_t)old * dim, 0, sizeof(double) * (size_t)(n - old) * dim, c->stream));
  }
  if (n != old) invalidate_graph(c);
  d->np = n;
  /* a new particle set starts per-particle Dormand-Prince from the context step */
  if (d->dopri_pp && n > 0) CU(cudaMemsetAsync(d->hp, 0, sizeof(double) * (size_t)n, c->stream));
  if (n > 0) {
    int i, *ones = (int *)malloc(sizeof(int) * (size_t)n);
    cudaError_t e = cudaSuccess;
    if (!ones) return set_error(LAGRBF_ERR_MEM, "out of host memory");
    for (i = 0; i < n; i++) ones[i] = 1;
    e = cudaMemcpyAsync(d->xp, coords, sizeof(double) * (size_t)n * dim, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess && values && F > 0)
      e = cudaMemcpyAsync(d->fields, values, sizeof(double) * (size_t)n * F, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(d->alive, ones, sizeof(int) * (size_t)n, cudaMemcpyHostToDevice, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    free(ones);
    if (e != cudaSuccess)
      return set_error(LAGRBF_ERR_GPU, "copying the particles to the device failed: %s", cudaGetErrorString(e));
  }
  OP(lgb_op_bin_particles(d, 1, c->stream));
  TRY(choose_chunk(c));
  CU(cudaStreamSynchronize(c->stream));
  c->points_filled = 1;
  return 0;
}

/* ---------------------------------------------------------------------------------------- */
/* interpolation                                                                            */
/* ---------------------------------------------------------------------------------------- */
static void prof_begin(lgb_ctx *c)
{
  if (c->profiling && c->nev < NPROF) cudaEventRecord(c->ev[2 * c->nev], c->stream);
}
static void prof_end(lgb_ctx *c)
{
  if (c->profiling && c->nev < NPROF) { cudaEventRecord(c->ev[2 * c->nev + 1], c->stream); c->nev++; }
}
static void prof_collect(lgb_ctx *c, double *acc)
{
  int i;
  if (!c->profiling || c->nev == 0) { c->nev = 0; return; }
  cudaStreamSynchronize(c->stream);
  for (i = 0; i < c->nev; i++) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, c->ev[2 * i], c->ev[2 * i + 1]);
    *acc += ms;
  }
  c->nev = 0;
}

static int eval_fields(lgb_ctx *c, int nf_first, int nf, double *out, int stride)
{
  int nl = (nf + 3) / 4;
  prof_begin(c);
  OP(lgb_op_eval(&c->d, nf_first, nf, out, stride, c->stream));
  prof_end(c);
  c->eval_launches += nl;
  return 0;
}

/* LagRBF_PartitionsSetUp: queue the patches touched by live particles, set up / solve them. */
static int partitions_setup(lgb_ctx *c)
{
  OP(lgb_op_mark_patches(&c->d, c->stream));
  if (c->profiling) {
    prof_collect(c, &c->eval_ms);
    cudaEventRecord(c->ev[0], c->stream);
  }
  OP(lgb_op_factor(&c->d, c->stream));
  OP(lgb_op_build_records(&c->d, 0, c->stream));
  if (c->profiling) {
    float ms = 0.f;
    cudaEventRecord(c->ev[1], c->stream);
    cudaStreamSynchronize(c->stream);
    cudaEventElapsedTime(&ms, c->ev[0], c->ev[1]);
    c->factor_ms += ms;
  }
  return 0;
}

static int check_factor_error(lgb_ctx *c)
{
  CU(cudaMemcpyAsync(c->hctrl, c->d.ctrl, sizeof(lgb_ctrl), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  if (c->hctrl->factor_error) {
    int row = c->hctrl->factor_error, node = c->hctrl->factor_node;
    CU(cudaMemsetAsync(&c->d.ctrl->factor_error, 0, sizeof(int), c->stream));
    return set_error(LAGRBF_ERR_MAT_CH_ZRPVT, "zero pivot in Cholesky factorisation of patch %d (row %d)", node, row);
  }
  return 0;
}

/* A bounded wait of the evaluation kernel that gave up (eval_error in the control block, read into
   hctrl by the caller): LAGRBF_ERR_TIMEOUT, and the flag is cleared so that the context stays
   usable for the next call. */
static int check_eval_error(lgb_ctx *c)
{
  if (!c->hctrl->eval_error) return 0;
  c->hctrl->eval_error = 0;
  CU(cudaMemsetAsync(&c->d.ctrl->eval_error, 0, sizeof(int), c->stream));
  CU(cudaStreamSynchronize(c->stream));
  return set_error(LAGRBF_ERR_TIMEOUT, "a bounded wait of the evaluation kernel gave up");
}

static int do_interpolation(lgb_ctx *c)
{
  lgb_dev *d = &c->d;
  if (!c->data_filled) return set_error(LAGRBF_ERR_ARG_WRONGSTATE, "data swarm is empty: fill the data first");
  if (!c->points_filled) return set_error(LAGRBF_ERR_ARG_WRONGSTATE, "interpolation swarm is empty: fill the points first");
  TRY(partitions_setup(c));
  TRY(check_factor_error(c));
  if (d->F > 0) TRY(eval_fields(c, 0, d->F, d->fields, d->F));
  prof_collect(c, &c->eval_ms);
  CU(cudaMemcpyAsync(c->hctrl, c->d.ctrl, sizeof(lgb_ctrl), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  TRY(check_eval_error(c));
  if (d->setup_all && !c->shared_from) c->all_ready = 1; /* every patch set up and solved */
  return 0;
}

static int reset_coefficients(lgb_ctx *c)
{
  lgb_dev *d = &c->d;
  if (c->shared_from) return 0; /* the patch set-ups belong to the dataset's owner */
  c->all_ready = 0;
  /* LagRBF_PartitionsReset: A_KSP_ASMB destroys the patch set-ups, the others only the solution */
  if (d->solve_method == LGB_A_KSP_ASMB) {
    CU(cudaMemsetAsync(d->setup, 0, sizeof(int) * (size_t)d->g.nnodes, c->stream));
    OP(lgb_op_build_records(d, 1, c->stream)); /* not-set-up patches contribute nothing */
  }
  CU(cudaMemsetAsync(d->solved, 0, sizeof(int) * (size_t)d->g.nnodes, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  return 0;
}

/* ---------------------------------------------------------------------------------------- */
/* advection                                                                                */
/* ---------------------------------------------------------------------------------------- */
static int host_velocity(lgb_ctx *c); /* analytical velocity through the user callback */

static int eval_velocity(lgb_ctx *c, int analytical)
{
  if (analytical) return host_velocity(c);
  return eval_fields(c, 0, c->d.g.dim, c->d.vel, c->d.g.dim);
}

/* One internal step of InternalForwardAdvectionLoop after the dt selection. */
static int step_sequence(lgb_ctx *c, int analytical)
{
  lgb_dev *d = &c->d;
  void *s = c->stream;
  int st;
  const int pp = (c->scheme == LGB_DOPRI && d->dopri_pp);
  OP(lgb_op_ctrl(d, pp ? LGB_CTRL_BEGIN_SWEEP : LGB_CTRL_BEGIN_STEP, s));
  switch (c->scheme) {
  case LGB_RK1:
    OP(lgb_op_stage(d, LGB_RK1, 0, s));
    OP(lgb_op_bin_particles(d, 1, s));
    break;
  case LGB_RK2:
    OP(lgb_op_stage(d, LGB_RK2, 0, s));
    OP(lgb_op_bin_particles(d, 1, s));
    TRY(eval_velocity(c, analytical));
    OP(lgb_op_stage(d, LGB_RK2, 1, s));
    OP(lgb_op_bin_particles(d, 1, s));
    break;
  case LGB_RK4:
    for (st = 0; st < 3; st++) {
      OP(lgb_op_stage(d, LGB_RK4, st, s));
      OP(lgb_op_bin_particles(d, 1, s));
      TRY(eval_velocity(c, analytical));
    }
    OP(lgb_op_stage(d, LGB_RK4, 3, s));
    OP(lgb_op_bin_particles(d, 1, s));
    break;
  case LGB_DOPRI:
    if (pp) {
      /* per-particle steps: only the particles still short of t_next are staged and evaluated */
      OP(lgb_op_pp_begin(d, s));
      for (st = 0; st < 6; st++) {
        OP(lgb_op_stage(d, LGB_DOPRI, st, s));
        OP(lgb_op_bin_particles_mask(d, 1, d->active, s));
        TRY(eval_velocity(c, analytical));
      }
      OP(lgb_op_pp_accept(d, s));
      OP(lgb_op_bin_particles(d, 1, s)); /* rejected particles are back at x0 */
      break;
    }
    for (st = 0; st < 6; st++) {
      OP(lgb_op_stage(d, LGB_DOPRI, st, s));
      OP(lgb_op_bin_particles(d, 1, s));
      TRY(eval_velocity(c, analytical));
    }
    OP(lgb_op_dopri_error(d, s));
    if (!c->reduce) OP(lgb_op_ctrl(d, LGB_CTRL_DOPRI_DT, s)); /* coupled runs: after the reduction */
    break;
  default:
    return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "unknown scheme");
  }
  if (!analytical) {
    TRY(partitions_setup(c));
    if (d->F > 0) TRY(eval_fields(c, 0, d->F, d->fields, d->F));
    OP(lgb_op_ctrl(d, LGB_CTRL_RESET_CFL, s));
    OP(lgb_op_copy_velocity(d, s));
  } else {
    TRY(host_velocity(c));
    OP(lgb_op_ctrl(d, LGB_CTRL_RESET_CFL, s));
    OP(lgb_op_count_alive(d, s));
  }
  OP(lgb_op_ctrl(d, pp ? LGB_CTRL_END_SWEEP : LGB_CTRL_END_STEP, s));
  return 0;
}

/* Coupled (sharded) runs: the step's local CFL step (from the largest |v|^2, as k_ctrl computes it)
   and DOPRI error are reduced over the ranks by the registered function, written back, and the
   DOPRI step update runs on the global error (the reference's MPI_Allreduce at advection.c:466 and
   dormand_prince.c:93).  hctrl holds the control block read after the step. */
static int couple_ranks(lgb_ctx *c, int dopri_update)
{
  lgb_ctrl *h = c->hctrl;
  double v[2], dt_cfl = DBL_MAX;
  int rc;
  if (h->n2max_bits) {
    double n2;
    unsigned long long b = h->n2max_bits - 1ull;
    memcpy(&n2, &b, sizeof n2);
    dt_cfl = h->cfl_fac * h->cfl_radius / (sqrt(n2) + 1e-16);
  }
  v[0] = -dt_cfl;
  v[1] = -DBL_MAX;
  if (dopri_update && h->any_alive) memcpy(&v[1], &h->maxerr_bits, sizeof(double));
  if ((rc = c->reduce(v, 2, c->ruser)))
    return set_error(LAGRBF_ERR_PLIB, "step reduction callback failed (%d)", rc);
  h->dt_cfl_ext = (-v[0] < DBL_MAX) ? -v[0] : 0.0;
  if (dopri_update) {
    h->any_alive = v[1] >= 0.0;
    if (h->any_alive) memcpy(&h->maxerr_bits, &v[1], sizeof(double));
  }
  CU(cudaMemcpyAsync(c->d.ctrl, h, sizeof(lgb_ctrl), cudaMemcpyHostToDevice, c->stream));
  if (dopri_update) OP(lgb_op_ctrl(&c->d, LGB_CTRL_DOPRI_DT, c->stream));
  CU(cudaMemcpyAsync(h, c->d.ctrl, sizeof(lgb_ctrl), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  return 0;
}

static int run_step(lgb_ctx *c, int analytical)
{
  /* the captured step differs between interpolated and device-field analytical advection */
  if (c->graph_valid && c->graph_mode != analytical) invalidate_graph(c);
  if ((analytical && !c->d.vfield) || c->profiling || !c->use_graph) {
    long long l0 = lgb_launch_count();
    TRY(step_sequence(c, analytical));
    c->launches_graph += 0;
    (void)l0;
    prof_collect(c, &c->eval_ms);
  } else if (c->graph_valid) {
    CU(cudaGraphLaunch(c->graph, c->stream));
    c->launches_graph += c->graph_launches;
    c->eval_launches += c->graph_eval_launches;
  } else {
    cudaGraph_t graph;
    long long l0 = lgb_launch_count(), e0 = c->eval_launches;
    cudaError_t e = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    int rc = 0;
    if (e == cudaSuccess) {
      rc = step_sequence(c, analytical);
      e = cudaStreamEndCapture(c->stream, &graph);
    }
    c->graph_eval_launches = c->eval_launches - e0;
    c->eval_launches = e0;
    if (e != cudaSuccess || rc) {
      /* capture not possible: run this step eagerly and stop using graphs */
      cudaGetLastError();
      c->use_graph = 0;
      TRY(step_sequence(c, analytical));
    } else {
      e = cudaGraphInstantiate(&c->graph, graph, 0);
      cudaGraphDestroy(graph);
      if (e != cudaSuccess) {
        cudaGetLastError();
        c->use_graph = 0;
        TRY(step_sequence(c, analytical));
      } else {
        c->graph_valid = 1;
        c->graph_mode = analytical;
        c->graph_launches = lgb_launch_count() - l0;
        /* the captured launches did not run; count them when the graph replays */
        c->launch_base += c->graph_launches;
        CU(cudaGraphLaunch(c->graph, c->stream));
        c->launches_graph += c->graph_launches;
        c->eval_launches += c->graph_eval_launches;
      }
    }
  }
  CU(cudaMemcpyAsync(c->hctrl, c->d.ctrl, sizeof(lgb_ctrl), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  if (c->hctrl->factor_error) return check_factor_error(c);
  TRY(check_eval_error(c));
  if (c->reduce && !(c->scheme == LGB_DOPRI && c->d.dopri_pp)) TRY(couple_ranks(c, c->scheme == LGB_DOPRI));
  return 0;
}

static int step_sequence(lgb_ctx *c, int analytical);

/* The internal steps of one advection interval as one graph launch: the step is the body of a
   conditional while node whose condition kernel continues while t < t_next (and no error flag is
   set, and at most loop_cap steps), so the host neither launches nor synchronises per step.
   Returns 1 when the interval was run this way, 0 when the caller must step from the host (coupled
   runs, host callbacks, profiling, graph capture off or not possible). */
static int run_interval_on_device(lgb_ctx *c, int analytical, int *rc)
{
  long long s0;
  *rc = 0;
  if (!c->use_graph || !c->device_loop || c->profiling || c->reduce || (analytical && !c->d.vfield) ||
      c->wgraph_failed)
    return 0;
  if (c->wgraph_valid && c->wgraph_mode != analytical) invalidate_graph(c);
  if (!c->wgraph_valid) {
    cudaGraph_t g = NULL, body;
    cudaGraphConditionalHandle h;
    struct cudaGraphNodeParams p;
    cudaGraphNode_t node;
    long long l0 = lgb_launch_count(), e0 = c->eval_launches;
    int ok = cudaGraphCreate(&g, 0) == cudaSuccess &&
             cudaGraphConditionalHandleCreate(&h, g, 1, cudaGraphCondAssignDefault) == cudaSuccess;
    if (ok) {
      memset(&p, 0, sizeof(p));
      p.type = cudaGraphNodeTypeConditional;
      p.conditional.handle = h;
      p.conditional.type = cudaGraphCondTypeWhile;
      p.conditional.size = 1;
      ok = cudaGraphAddNode(&node, g, NULL, NULL, 0, &p) == cudaSuccess;
    }
    if (ok) {
      body = p.conditional.phGraph_out[0];
      ok = cudaStreamBeginCaptureToGraph(c->stream, body, NULL, NULL, 0, cudaStreamCaptureModeThreadLocal) ==
           cudaSuccess;
      if (ok) {
        int r = step_sequence(c, analytical);
        if (!r) r = lgb_op_loop_cond(&c->d, (unsigned long long)h, c->stream);
        ok = (cudaStreamEndCapture(c->stream, &body) == cudaSuccess) && !r;
        /* a capture into the conditional body that failed leaves that body in no defined state:
           destroying the parent graph then crashed the driver, so this one graph is left alone
           (once per context: the device loop is off from then on) */
        if (!ok) g = NULL;
      }
    }
    c->wgraph_eval_launches = c->eval_launches - e0;
    c->eval_launches = e0;
    c->wgraph_launches = lgb_launch_count() - l0;
    c->launch_base += c->wgraph_launches; /* captured, not run */
    if (ok) ok = cudaGraphInstantiate(&c->wgraph, g, 0) == cudaSuccess;
    if (g) cudaGraphDestroy(g);
    if (!ok) {
      cudaGetLastError();
      c->wgraph_failed = 1; /* keep stepping from the host */
      return 0;
    }
    c->wgraph_valid = 1;
    c->wgraph_mode = analytical;
  }
  s0 = c->hctrl->steps;
  CU(cudaGraphLaunch(c->wgraph, c->stream));
  CU(cudaMemcpyAsync(c->hctrl, c->d.ctrl, sizeof(lgb_ctrl), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  c->launches_graph += (c->hctrl->steps - s0) * c->wgraph_launches;
  c->eval_launches += (c->hctrl->steps - s0) * c->wgraph_eval_launches;
  if (c->hctrl->factor_error) *rc = check_factor_error(c);
  else *rc = check_eval_error(c);
  return 1;
}

static int advection_loop(lgb_ctx *c, double t, double t_next, int analytical, int keep)
{
  lgb_dev *d = &c->d;
  int it = 0;
  if (!c->points_filled) return set_error(LAGRBF_ERR_ARG_WRONGSTATE, "swarm to advect has not been provided");
  if (!analytical && !c->data_filled) return set_error(LAGRBF_ERR_ARG_WRONGSTATE, "data swarm is empty: fill the data first");
  if (!analytical && d->F < d->g.dim)
    return set_error(LAGRBF_ERR_ARG_SIZ, "advection needs n_interpolation_fields >= dim (velocity = first dim fields)");
  /* loop scalars into the control block */
  CU(cudaMemcpyAsync(c->hctrl, d->ctrl, sizeof(lgb_ctrl), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  c->hctrl->t = t;
  c->hctrl->t_next = t_next;
  c->hctrl->scheme = c->scheme;
  c->hctrl->pp_hmin = 1e-10 * (t_next - t);
  c->hctrl->loop_iter = 0;
  c->hctrl->loop_cap = 1 << 20;
  CU(cudaMemcpyAsync(d->ctrl, c->hctrl, sizeof(lgb_ctrl), cudaMemcpyHostToDevice, c->stream));
  /* AdvectionInitializeTimestepVelocity, then the CFL of that velocity */
  OP(lgb_op_ctrl(d, LGB_CTRL_RESET_CFL, c->stream));
  if (analytical) {
    TRY(host_velocity(c));
    OP(lgb_op_count_alive(d, c->stream));
  } else {
    OP(lgb_op_copy_velocity(d, c->stream));
  }
  if (c->scheme == LGB_DOPRI && d->dopri_pp) OP(lgb_op_pp_init(d, t, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  if (c->reduce && !(c->scheme == LGB_DOPRI && d->dopri_pp)) {
    CU(cudaMemcpyAsync(c->hctrl, d->ctrl, sizeof(lgb_ctrl), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    TRY(couple_ranks(c, 0)); /* the first step's CFL step over all ranks */
  }
  if (t < t_next) {
    int rc;
    if (run_interval_on_device(c, analytical, &rc)) {
      TRY(rc);
      t = c->hctrl->t; /* beyond the iteration limit the host continues step by step */
    }
  }
  while (t < t_next) {
    TRY(run_step(c, analytical));
    t = c->hctrl->t;
    it++;
  }
  if (!analytical && !keep) {
    /* end of the time step (time_loop.c:93-98): reset partitions, cell info, clear the data swarm */
    TRY(reset_coefficients(c));
    c->data_filled = 0;
  }
  return 0;
}

static int host_velocity(lgb_ctx *c)
{
  /* AdvectionEvaluateVelocityFunction (advection.c:318-351): the callback sees the live
     particles packed contiguously, like the swarm after migration.  A device-side field, when set,
     replaces the callback and stays on the stream. */
  lgb_dev *d = &c->d;
  int dim = d->g.dim, n = d->np, p, q = 0, nl = 0, rc = 0;
  double *x = NULL, *v = NULL, *xc = NULL, *vc = NULL;
  int *alive = NULL;
  if (n == 0) return 0;
  if (d->vfield) {
    OP(lgb_op_velocity_field(d, c->stream));
    return 0;
  }
  x = (double *)malloc(sizeof(double) * (size_t)n * dim);
  v = (double *)malloc(sizeof(double) * (size_t)n * dim);
  xc = (double *)malloc(sizeof(double) * (size_t)n * dim);
  vc = (double *)calloc((size_t)n * dim, sizeof(double));
  alive = (int *)malloc(sizeof(int) * (size_t)n);
  if (!x || !v || !xc || !vc || !alive) { rc = set_error(LAGRBF_ERR_MEM, "out of host memory"); goto done; }
  if (cudaMemcpyAsync(x, d->xp, sizeof(double) * (size_t)n * dim, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaMemcpyAsync(v, d->vel, sizeof(double) * (size_t)n * dim, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaMemcpyAsync(alive, d->alive, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess) {
    rc = set_error(LAGRBF_ERR_GPU, "copying particles to the host failed");
    goto done;
  }
  for (p = 0; p < n; p++) if (alive[p]) { memcpy(&xc[(size_t)nl * dim], &x[(size_t)p * dim], sizeof(double) * dim); nl++; }
  if (c->vfnb) rc = c->vfnb(nl, dim, xc, vc, c->vuser);
  else if (c->vfn) for (q = 0; q < nl && !rc; q++) rc = c->vfn(&xc[(size_t)q * dim], &vc[(size_t)q * dim], c->vuser);
  else rc = set_error(LAGRBF_ERR_ARG_NULL, "no velocity function registered");
  if (rc) { rc = set_error(rc, "velocity callback returned %d", rc); goto done; }
  q = 0;
  for (p = 0; p < n; p++) if (alive[p]) { memcpy(&v[(size_t)p * dim], &vc[(size_t)q * dim], sizeof(double) * dim); q++; }
  if (cudaMemcpyAsync(d->vel, v, sizeof(double) * (size_t)n * dim, cudaMemcpyHostToDevice, c->stream) != cudaSuccess ||
      cudaStreamSynchronize(c->stream) != cudaSuccess)
    rc = set_error(LAGRBF_ERR_GPU, "copying velocities to the device failed");
done:
  free(x); free(v); free(xc); free(vc); free(alive);
  return rc;
}

/* ---------------------------------------------------------------------------------------- */
/* output                                                                                   */
/* ---------------------------------------------------------------------------------------- */
static int do_output(lgb_ctx *c, int is_data, int nglobal, double *coords, double *fields, int64_t *pidx,
                     const char *fieldname)
{
  lgb_dev *d = &c->d;
  int dim = d->g.dim, n = is_data ? d->nd : d->np, nf = 0, p, f, rc = 0;
  const int64_t *pid = is_data ? c->pid_d : c->pid_p;
  double *hx = NULL, *hf = NULL, *wtmp = NULL;
  int *alive = NULL;
  const double *src = NULL;
  if (nglobal < 0) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "negative npoints");
  if (fields) {
    if (!fieldname || strcmp(fieldname, "fields") == 0) { src = is_data ? d->fd : d->fields; nf = d->F; }
    else if (!is_data && strcmp(fieldname, "velocity") == 0) { src = d->vel; nf = dim; }
    else if (!is_data && strcmp(fieldname, "weights") == 0) {
      int err = 0;
      nf = d->g.nen;
      wtmp = (double *)dalloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * nf, &err);
      if (err) return set_error(LAGRBF_ERR_MEM, "weights buffer allocation failed");
      CU(cudaMemsetAsync(wtmp, 0, sizeof(double) * (size_t)(n > 0 ? n : 1) * nf, c->stream));
      OP(lgb_op_weights(d, wtmp, c->stream));
      src = wtmp;
    } else return set_error(LAGRBF_ERR_ARG_WRONG, "unknown field \"%s\"", fieldname);
  }
  if (!is_data && c->out_direct) {
    /* the GPU writes every output row into the caller's arrays (pid order, zero rows for pids no
       longer in the swarm) */
    int err = 0, bad = 0;
    if (n > c->pidd_cap) {
      DFREE(c->pidd);
      c->pidd = (long long *)dalloc(sizeof(long long) * (size_t)n, &err);
      c->pidd_cap = err ? 0 : n;
      c->pidd_valid = 0;
    }
    if (!c->pidd_valid && n > 0 && !err) {
      CU(cudaMemcpyAsync(c->pidd, c->pid_p, sizeof(long long) * (size_t)n, cudaMemcpyHostToDevice, c->stream));
      c->pidd_valid = 1;
    }
    if (!err && (long long)nglobal > c->out_inv_cap) {
      DFREE(c->out_inv);
      c->out_inv = (int *)dalloc(sizeof(int) * (size_t)(nglobal > 0 ? nglobal : 1), &err);
      c->out_inv_cap = err ? 0 : nglobal;
    }
    if (!err && !c->out_bad) c->out_bad = (int *)dalloc(sizeof(int), &err);
    if (err) { rc = set_error(LAGRBF_ERR_MEM, "output scratch allocation failed"); goto done; }
    OP(lgb_op_output_rows(n, c->pidd, d->alive, nglobal, c->out_inv, c->out_bad, dim, d->xp, coords, nf, src, fields,
                          (long long *)pidx, d->nsm, c->stream));
    CU(cudaMemcpyAsync(&bad, c->out_bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    if (bad) rc = set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "a particle pid is out of range [1, %d]", nglobal);
    goto done;
  }
  hx = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * dim);
  hf = (double *)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * (nf > 0 ? nf : 1));
  alive = (int *)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  if (!hx || !hf || !alive) { rc = set_error(LAGRBF_ERR_MEM, "out of host memory"); goto done; }
  if (n > 0) {
    cudaMemcpyAsync(hx, is_data ? d->xd : d->xp, sizeof(double) * (size_t)n * dim, cudaMemcpyDeviceToHost, c->stream);
    if (src && nf > 0) cudaMemcpyAsync(hf, src, sizeof(double) * (size_t)n * nf, cudaMemcpyDeviceToHost, c->stream);
    if (!is_data) cudaMemcpyAsync(alive, d->alive, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost, c->stream);
    if (cudaStreamSynchronize(c->stream) != cudaSuccess) { rc = set_error(LAGRBF_ERR_GPU, "device to host copy failed"); goto done; }
  }
  /* AssembleArray_Allreduce (interface_utils.c:188-263): zero, then scatter by pid - 1 */
  if (coords) memset(coords, 0, sizeof(double) * (size_t)nglobal * dim);
  if (fields) memset(fields, 0, sizeof(double) * (size_t)nglobal * nf);
  if (pidx) memset(pidx, 0, sizeof(int64_t) * (size_t)nglobal);
  for (p = 0; p < n; p++) {
    int64_t gi;
    if (!is_data && !alive[p]) continue;
    gi = pid[p] - 1;
    if (gi < 0 || gi >= nglobal) {
      rc = set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "pid %lld out of range [0, %d)", (long long)gi, nglobal);
      goto done;
    }
    if (coords) for (f = 0; f < dim; f++) coords[gi * dim + f] = hx[(size_t)p * dim + f];
    if (fields) for (f = 0; f < nf; f++) fields[gi * nf + f] = hf[(size_t)p * nf + f];
    if (pidx) pidx[gi] = pid[p];
  }
done:
  free(hx); free(hf); free(alive);
  if (wtmp) cudaFree(wtmp);
  return rc;
}

/* ======================================================================================= */
/* section 1: the drop-in surface                                                           */
/* ======================================================================================= */
LAGRBF_EXPORT void *lagrbf_create(void)
{
  lgb_ctx *c = NULL;
  if (create_ctx(&c)) return NULL;
  return c;
}

LAGRBF_EXPORT void lagrbf_destroy(void *ctx)
{
  if (ctx) destroy_ctx((lgb_ctx *)ctx);
}

LAGRBF_EXPORT int lagrbf_fill_swarm(void *ctx, bool is_data, int32_t npoints, double *coords, double *values,
                                    int64_t *pidx)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  if (npoints < 0) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "negative npoints");
  if (npoints > 0 && !coords) return set_error(LAGRBF_ERR_ARG_NULL, "coords is NULL");
  return is_data ? fill_data(c, npoints, coords, values, pidx) : fill_points(c, npoints, coords, values, pidx);
}

LAGRBF_EXPORT int lagrbf_interpolation(void *ctx)
{
  if (!ctx) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  return do_interpolation((lgb_ctx *)ctx);
}

LAGRBF_EXPORT int lagrbf_output(void *ctx, bool is_data, int32_t npoints, double *coords, double *fields,
                                int64_t *pidx, const char *fieldname)
{
  if (!ctx) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  return do_output((lgb_ctx *)ctx, is_data, npoints, coords, fields, pidx, fieldname);
}

LAGRBF_EXPORT int lagrbf_reset_coefficients(void *ctx)
{
  if (!ctx) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  return reset_coefficients((lgb_ctx *)ctx);
}

LAGRBF_EXPORT int lagrbf_avect_analytical(void *ctx, double time, double time_next)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "LagRBFCtx is NULL");
  if (!c->vfn && !c->vfnb && !c->d.vfield) return set_error(LAGRBF_ERR_ARG_NULL, "no velocity function registered");
  return advection_loop(c, time, time_next, 1, 0);
}

LAGRBF_EXPORT int lagrbf_advect_interpolate(void *ctx, double time, double time_next)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "LagRBFCtx is NULL");
  if (c->vfn || c->vfnb) return set_error(LAGRBF_ERR_ARG_WRONGSTATE, "an analytical velocity function is registered");
  return advection_loop(c, time, time_next, 0, 0);
}

LAGRBF_EXPORT int lagrbf_advection_function(void *ctx, int (*velocity_fn)(double *, double *, void *), void *fn_ctx)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  c->vfn = velocity_fn;
  c->vuser = fn_ctx;
  return 0;
}

LAGRBF_EXPORT int lagrbf_advection_function_batch(void *ctx,
                                                  int (*velocity_fn_batch)(int32_t, int32_t, double *, double *, void *),
                                                  void *fn_ctx)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  c->vfnb = velocity_fn_batch;
  c->vuser = fn_ctx;
  return 0;
}

LAGRBF_EXPORT void lagrbf_interpolate_driver(int32_t ndata_local, double *data_coords, double *data_values,
                                             int32_t npoints_local, double *points_coords, double *points_values,
                                             int32_t npoints_global, char *options_file)
{
  lgb_ctx *c = NULL;
  int rc = 0;
  if (options_file && options_file[0]) rc = lagrbf_options_insert_file(options_file);
  if (!rc) rc = create_ctx(&c);
  if (!rc) rc = fill_data(c, ndata_local, data_coords, data_values, NULL);
  if (!rc) rc = fill_points(c, npoints_local, points_coords, NULL, NULL);
  if (!rc) rc = do_interpolation(c);
  if (!rc) rc = do_output(c, 0, npoints_global, NULL, points_values, NULL, "fields");
  if (rc) fprintf(stderr, "ERROR: lagrbf_interpolate() failed with error code %d: %s\n", rc, g_errmsg);
  if (c) destroy_ctx(c);
}

/* ======================================================================================= */
/* section 3: GPU-level extension                                                           */
/* ======================================================================================= */
LAGRBF_EXPORT int lagrbf_gpu_advect_resident(void *ctx, double time, double time_next)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "LagRBFCtx is NULL");
  if (c->vfn || c->vfnb) return set_error(LAGRBF_ERR_ARG_WRONGSTATE, "an analytical velocity function is registered");
  return advection_loop(c, time, time_next, 0, 1);
}

double lgb_fp32_peak_tflops(void);
LAGRBF_EXPORT double lagrbf_gpu_fp32_peak_tflops(void) { return lgb_fp32_peak_tflops(); }
double lgb_fp64_peak_tflops(void);
LAGRBF_EXPORT double lagrbf_gpu_fp64_peak_tflops(void) { return lgb_fp64_peak_tflops(); }

LAGRBF_EXPORT int lagrbf_gpu_set_velocity_field(void *ctx, int32_t kind, const double *params, int32_t nparams)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  lgb_dev *d;
  int need = 0, err = 0;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  d = &c->d;
  switch (kind) {
  case LGB_VF_NONE: need = 0; break;
  case LGB_VF_ROTATION: need = 3; break;
  case LGB_VF_CELLULAR: need = 2; break;
  case LGB_VF_ABC: need = 4; break;
  case LGB_VF_FOURIER:
    if (nparams < 1 || !params) return set_error(LAGRBF_ERR_ARG_SIZ, "Fourier field: parameters missing");
    if (!(params[0] >= 0.0) || params[0] > 4096.0) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "Fourier field: bad mode count");
    need = 1 + 7 * (int)params[0];
    break;
  default: return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "unknown velocity field kind %d", kind);
  }
  if (nparams < need || (need > 0 && !params))
    return set_error(LAGRBF_ERR_ARG_SIZ, "velocity field kind %d needs %d parameters, got %d", kind, need, nparams);
  CU(cudaStreamSynchronize(c->stream));
  DFREE(d->vfield_par);
  d->vfield = 0;
  d->vfield_np = 0;
  if (kind != LGB_VF_NONE) {
    d->vfield_par = (double *)dalloc(sizeof(double) * (size_t)(need > 0 ? need : 1), &err);
    if (err) return set_error(LAGRBF_ERR_MEM, "velocity field parameters allocation failed");
    if (need > 0) CU(cudaMemcpy(d->vfield_par, params, sizeof(double) * (size_t)need, cudaMemcpyHostToDevice));
    d->vfield = kind;
    d->vfield_np = need;
  }
  invalidate_graph(c);
  return 0;
}

LAGRBF_EXPORT int lagrbf_gpu_set_precision(void *ctx, int fp32)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  CU(cudaStreamSynchronize(c->stream));
  c->d.prec = fp32 ? LGB_PREC_FP32 : LGB_PREC_FP64;
  invalidate_graph(c);
  return 0;
}

LAGRBF_EXPORT int lagrbf_gpu_share_dataset(void *ctx, void *owner)
{
  lgb_ctx *c = (lgb_ctx *)ctx, *o = (lgb_ctx *)owner;
  lgb_dev *d;
  int k;
  if (!c || !o) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  d = &c->d;
  if (c == o || c->shared_from || o->shared_from)
    return set_error(LAGRBF_ERR_ARG_WRONGSTATE, "dataset sharing: one owner, one level of sharing");
  if (!o->data_filled || !o->all_ready)
    return set_error(LAGRBF_ERR_ARG_WRONGSTATE,
                     "dataset sharing: the owner needs setup_all_patches and a completed interpolation");
  if (c->data_filled || d->nd > 0) return set_error(LAGRBF_ERR_ARG_WRONGSTATE, "dataset sharing: ctx has its own data");
  if (d->g.dim != o->d.g.dim || d->g.kernel != o->d.g.kernel || d->F != o->d.F || d->g.eps_r != o->d.g.eps_r ||
      d->g.eps_w != o->d.g.eps_w || d->solve_method != o->d.solve_method)
    return set_error(LAGRBF_ERR_ARG_WRONG, "dataset sharing: different mesh, kernel or fields");
  for (k = 0; k < 3; k++)
    if (d->g.n[k] != o->d.g.n[k] || d->g.O[k] != o->d.g.O[k] || d->g.L[k] != o->d.g.L[k])
      return set_error(LAGRBF_ERR_ARG_WRONG, "dataset sharing: different PU mesh");
  /* The owner's stream is not synchronised here: all_ready is set only after the owner's
     interpolation has drained that stream, and the owner's thread may be capturing a graph on it
     right now (a synchronisation from this thread would invalidate that capture). */
  CU(cudaStreamSynchronize(c->stream));
  free_data(d);
  DFREE(d->cstart); DFREE(d->pm); DFREE(d->slot); DFREE(d->setup); DFREE(d->solved);
  DFREE(d->coff); DFREE(d->foff); DFREE(d->c64); DFREE(d->c32); DFREE(d->fac); DFREE(d->rec32); DFREE(d->rec_off);
  borrow_dataset(d, &o->d);
  d->setup_all = 1; /* every patch of the borrowed dataset is set up: nothing is queued */
  c->shared_from = o;
  c->data_filled = 1;
  invalidate_graph(c);
  return 0;
}

LAGRBF_EXPORT int lagrbf_gpu_set_step_reduce(void *ctx, int (*fn)(double *, int32_t, void *), void *user)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  CU(cudaStreamSynchronize(c->stream));
  c->reduce = fn;
  c->ruser = user;
  if (!fn) {
    c->hctrl->dt_cfl_ext = 0.0;
    CU(cudaMemcpy(&c->d.ctrl->dt_cfl_ext, &c->hctrl->dt_cfl_ext, sizeof(double), cudaMemcpyHostToDevice));
  }
  invalidate_graph(c);
  return 0;
}

LAGRBF_EXPORT int lagrbf_gpu_test_eval_wait(void *ctx, int32_t poll_limit, int32_t withhold_copies)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  if (poll_limit < 0) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "poll limit must be >= 0");
  CU(cudaStreamSynchronize(c->stream));
  c->d.eval_poll_limit = poll_limit;
  c->d.eval_withhold = withhold_copies ? 1 : 0;
  invalidate_graph(c);
  return 0;
}

LAGRBF_EXPORT int lagrbf_gpu_set_profiling(void *ctx, int on)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  c->profiling = on ? 1 : 0;
  if (on) invalidate_graph(c);
  return 0;
}

static int cmp_double(const void *a, const void *b)
{
  const double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

LAGRBF_EXPORT int lagrbf_gpu_set_condition_estimates(void *ctx, int on)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  lgb_dev *d;
  int err = 0;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  d = &c->d;
  CU(cudaStreamSynchronize(c->stream));
  if (on && !d->kappa) {
    d->kappa = (double *)dalloc(sizeof(double) * (size_t)d->g.nnodes, &err);
    if (err) return set_error(LAGRBF_ERR_MEM, "condition estimate array allocation failed");
    CU(cudaMemset(d->kappa, 0, sizeof(double) * (size_t)d->g.nnodes));
  }
  d->cond_on = on ? 1 : 0;
  invalidate_graph(c);
  return 0;
}

/* Condition estimates of the patches factored since they were switched on (0 where none). */
LAGRBF_EXPORT int lagrbf_gpu_get_condition(void *ctx, double *kappa, double *summary)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  int nn, i, n = 0;
  double *k;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  if (summary) summary[0] = summary[1] = summary[2] = 0.0;
  if (!c->d.kappa) return 0;
  nn = c->d.g.nnodes;
  k = (double *)malloc(sizeof(double) * (size_t)nn);
  if (!k) return set_error(LAGRBF_ERR_MEM, "out of host memory");
  CU(cudaStreamSynchronize(c->stream));
  CUF(cudaMemcpy(k, c->d.kappa, sizeof(double) * (size_t)nn, cudaMemcpyDeviceToHost), free(k));
  if (kappa) memcpy(kappa, k, sizeof(double) * (size_t)nn);
  for (i = 0; i < nn; i++)
    if (k[i] > 0.0) k[n++] = k[i];
  if (summary && n > 0) {
    qsort(k, (size_t)n, sizeof(double), cmp_double);
    summary[0] = k[n - 1];
    summary[1] = (n & 1) ? k[n / 2] : 0.5 * (k[n / 2 - 1] + k[n / 2]);
    summary[2] = n;
  }
  free(k);
  return 0;
}

LAGRBF_EXPORT int lagrbf_gpu_get_stats(void *ctx, lagrbf_stats_t *st)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  int nn, *setup, i, ns = 0;
  if (!c || !st) return set_error(LAGRBF_ERR_ARG_NULL, "NULL argument");
  CU(cudaMemcpyAsync(c->hctrl, c->d.ctrl, sizeof(lgb_ctrl), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  nn = c->d.g.nnodes;
  setup = (int *)malloc(sizeof(int) * (size_t)nn);
  if (setup) {
    CUF(cudaMemcpy(setup, c->d.setup, sizeof(int) * (size_t)nn, cudaMemcpyDeviceToHost), free(setup));
    for (i = 0; i < nn; i++) ns += setup[i] != 0;
    free(setup);
  }
  memset(st, 0, sizeof(*st));
  st->launches = lgb_launch_count() - c->launch_base + c->launches_graph;
  st->eval_launches = c->eval_launches;
  st->eval_flops = c->hctrl->eval_flops;
  st->eval_bytes = c->hctrl->eval_bytes;
  st->eval_ms = c->eval_ms;
  st->particle_steps = c->hctrl->particle_steps;
  st->steps = c->hctrl->steps;
  st->patches_factored = c->hctrl->nfactored;
  st->factor_ms = c->factor_ms;
  st->factor_flops = c->hctrl->factor_flops;
  st->np_alive = c->hctrl->np_alive;
  st->nd = c->d.nd;
  st->max_patch = c->d.max_patch;
  st->npatch_setup = ns;
  st->dt = c->hctrl->dt_adv;
  st->chunk_cap = c->d.chunk_cap;
  st->records = c->d.rec32 != NULL;
  st->device_loop = c->wgraph_valid;
  if (c->d.cond_on) {
    double sm[3];
    TRY(lagrbf_gpu_get_condition(ctx, NULL, sm));
    st->kappa_max = sm[0];
    st->kappa_median = sm[1];
  }
  return 0;
}

LAGRBF_EXPORT int lagrbf_gpu_reset_stats(void *ctx)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  CU(cudaStreamSynchronize(c->stream));
  CU(cudaMemcpy(c->hctrl, c->d.ctrl, sizeof(lgb_ctrl), cudaMemcpyDeviceToHost));
  c->hctrl->eval_flops = 0.0;
  c->hctrl->eval_bytes = 0.0;
  c->hctrl->particle_steps = 0;
  c->hctrl->steps = 0;
  c->hctrl->nfactored = 0;
  c->hctrl->factor_flops = 0.0;
  CU(cudaMemcpy(c->d.ctrl, c->hctrl, sizeof(lgb_ctrl), cudaMemcpyHostToDevice));
  c->eval_ms = 0.0;
  c->factor_ms = 0.0;
  c->eval_launches = 0;
  c->launches_graph = 0;
  c->launch_base = lgb_launch_count();
  return 0;
}

LAGRBF_EXPORT int lagrbf_gpu_synchronize(void *ctx)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  CU(cudaStreamSynchronize(c->stream));
  return 0;
}

LAGRBF_EXPORT void *lagrbf_gpu_stream(void *ctx) { return ctx ? (void *)((lgb_ctx *)ctx)->stream : NULL; }

LAGRBF_EXPORT int lagrbf_gpu_get_cellids(void *ctx, bool is_data, int32_t *cellid)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  int n;
  if (!c || !cellid) return set_error(LAGRBF_ERR_ARG_NULL, "NULL argument");
  n = is_data ? c->d.nd : c->d.np;
  if (n > 0) CU(cudaMemcpy(cellid, is_data ? c->d.cell_d : c->d.cell_p, sizeof(int) * (size_t)n, cudaMemcpyDeviceToHost));
  return 0;
}

/* Patch membership in the reference's data order (partition.c:337-371), as data (fill) indices. */
LAGRBF_EXPORT int64_t lagrbf_gpu_get_patch_csr(void *ctx, int32_t *patch_start, int32_t *patch_pts)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  lgb_dev *d;
  int nn, nc, nd, i, s;
  int *cstart, *sorted;
  long long total = 0;
  cudaError_t e;
  if (!c) return -set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  d = &c->d;
  nn = d->g.nnodes; nc = d->g.ncells; nd = d->nd;
  cstart = (int *)malloc(sizeof(int) * (size_t)(nc + 1));
  sorted = (int *)malloc(sizeof(int) * (size_t)(nd > 0 ? nd : 1));
  if (!cstart || !sorted) { free(cstart); free(sorted); return -set_error(LAGRBF_ERR_MEM, "out of host memory"); }
  e = cudaMemcpy(cstart, d->cstart, sizeof(int) * (size_t)(nc + 1), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && nd > 0) e = cudaMemcpy(sorted, d->sorted, sizeof(int) * (size_t)nd, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    free(cstart); free(sorted);
    return -set_error(LAGRBF_ERR_GPU, "copying the cell lists failed: %s", cudaGetErrorString(e));
  }
  for (i = 0; i < nn; i++) {
    int nxy = d->g.n[0] * d->g.n[1], l = i / nxy, r = i - l * nxy, j = r / d->g.n[0], ii = r - j * d->g.n[0];
    if (patch_start) patch_start[i] = (int)total;
    for (s = 0; s < 8; s++) {
      int dx = s & 1, dy = (s >> 1) & 1, dz = (s >> 2) & 1, ci = ii - 1 + dx, cj = j - 1 + dy;
      int cl = (d->g.dim == 3) ? l - 1 + dz : 0, cc, q;
      if (d->g.dim == 2 && dz) continue;
      if (ci < 0 || ci >= d->g.nc[0] || cj < 0 || cj >= d->g.nc[1] || cl < 0 || cl >= d->g.nc[2]) continue;
      cc = ci + cj * d->g.nc[0] + cl * d->g.nc[0] * d->g.nc[1];
      for (q = cstart[cc]; q < cstart[cc + 1]; q++) {
        if (patch_pts) patch_pts[total] = sorted[q];
        total++;
      }
    }
  }
  if (patch_start) patch_start[nn] = (int)total;
  free(cstart); free(sorted);
  return total;
}

LAGRBF_EXPORT int64_t lagrbf_gpu_get_block_csr(void *ctx, int32_t *blk_start, int32_t *blk_pts)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  lgb_dev *d;
  int nc, nd, cell;
  int *cstart, *sorted;
  long long total = 0;
  cudaError_t e;
  if (!c) return -set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  d = &c->d;
  nc = d->g.ncells; nd = d->nd;
  cstart = (int *)malloc(sizeof(int) * (size_t)(nc + 1));
  sorted = (int *)malloc(sizeof(int) * (size_t)(nd > 0 ? nd : 1));
  if (!cstart || !sorted) { free(cstart); free(sorted); return -set_error(LAGRBF_ERR_MEM, "out of host memory"); }
  e = cudaMemcpy(cstart, d->cstart, sizeof(int) * (size_t)(nc + 1), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && nd > 0) e = cudaMemcpy(sorted, d->sorted, sizeof(int) * (size_t)nd, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) {
    free(cstart); free(sorted);
    return -set_error(LAGRBF_ERR_GPU, "copying the cell lists failed: %s", cudaGetErrorString(e));
  }
  for (cell = 0; cell < nc; cell++) {
    int cx = d->g.nc[0], cy = d->g.nc[1], cz = d->g.nc[2];
    int l = cell / (cx * cy), j = (cell - l * cx * cy) / cx, i = cell - l * cx * cy - j * cx, dz, dy, dx;
    int zlo = (d->g.dim == 3) ? -1 : 0, zhi = (d->g.dim == 3) ? 1 : 0;
    if (blk_start) blk_start[cell] = (int)total;
    for (dz = zlo; dz <= zhi; dz++)
      for (dy = -1; dy <= 1; dy++)
        for (dx = -1; dx <= 1; dx++) {
          int ii = i + dx, jj = j + dy, ll = l + dz, nb, q;
          if (ii < 0 || ii >= cx || jj < 0 || jj >= cy || ll < 0 || ll >= cz) continue;
          nb = ii + jj * cx + ll * cx * cy;
          for (q = cstart[nb]; q < cstart[nb + 1]; q++) {
            if (blk_pts) blk_pts[total] = sorted[q];
            total++;
          }
        }
  }
  if (blk_start) blk_start[nc] = (int)total;
  free(cstart); free(sorted);
  return total;
}

LAGRBF_EXPORT int lagrbf_gpu_get_geometry(void *ctx, int32_t *ints, double *reals)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c || !ints || !reals) return set_error(LAGRBF_ERR_ARG_NULL, "NULL argument");
  ints[0] = c->d.g.dim; ints[1] = c->d.g.n[0]; ints[2] = c->d.g.n[1]; ints[3] = c->d.g.n[2];
  ints[4] = c->d.g.nnodes; ints[5] = c->d.g.ncells; ints[6] = c->d.g.nen;
  reals[0] = c->d.g.eps_w; reals[1] = c->d.g.eps_r;
  return 0;
}

int lgb_ctx_dims(void *ctx, int *dim, int *nfields)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  *dim = c->d.g.dim;
  *nfields = c->d.F;
  return 0;
}

/* Scheme, initial step and CFL factor of an existing context (the serving loop runs jobs with
   different RK orders and steps on one resident dataset, and reuses contexts between jobs). */
int lgb_ctx_set_scheme(void *ctx, int scheme, double dt, double cfl)
{
  lgb_ctx *c = (lgb_ctx *)ctx;
  if (!c) return set_error(LAGRBF_ERR_ARG_NULL, "context is NULL");
  if (scheme < 0 || scheme > 3) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "unknown advection scheme %d", scheme);
  if (!(cfl > 0.0)) return set_error(LAGRBF_ERR_ARG_OUTOFRANGE, "CFL factor must be positive");
  CU(cudaMemcpyAsync(c->hctrl, c->d.ctrl, sizeof(lgb_ctrl), cudaMemcpyDeviceToHost, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  c->scheme = scheme;
  c->dt0 = dt;
  c->cfl_fac = cfl;
  c->hctrl->scheme = scheme;
  c->hctrl->cfl_fac = cfl;
  c->hctrl->dt_adv = dt;
  c->hctrl->dopri_error = DBL_MAX;
  CU(cudaMemcpyAsync(c->d.ctrl, c->hctrl, sizeof(lgb_ctrl), cudaMemcpyHostToDevice, c->stream));
  CU(cudaStreamSynchronize(c->stream));
  invalidate_graph(c);
  return 0;
}
