/*
 * lgb_serve.c -- serving loop: advection jobs admitted by device-memory budget, run concurrently.
 *
 * No counterpart in the reference (one application run per PETSc job there).  A job is a dataset
 * (nodal field on scattered points, or the id of a resident dataset), a particle set, an RK order
 * and a number of steps.  Worker threads take jobs from a FIFO queue as soon as the device-memory
 * budget and the job's dataset allow, each job on its own context (its own CUDA stream, its own
 * captured step graph), so jobs that arrive while others run are admitted as memory frees up and
 * their work overlaps on the device.  Datasets with an id stay resident after their job (data,
 * every patch set up and solved, coefficients, record blocks): a later job on the same id skips
 * the set-up, and jobs on a dataset whose context is busy run at the same time on contexts that
 * share it read-only (lagrbf_gpu_share_dataset).  Idle resident datasets are evicted, least
 * recently used first, when a job needs their memory.
 *
 * The server is a client of the context API of this library (lagrbf_create ... lagrbf_output);
 * a job's result is its particle positions after the last step, by pid.
 */
#include "lgb_internal.h"
#include "../../include/lagrbf.h"

#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

int lgb_set_error_msg(int code, const char *msg);
int lgb_ctx_set_scheme(void *ctx, int scheme, double dt, double cfl);

/* Device bytes of a context that shares a resident dataset, beyond its particles. */
#define SHARE_BYTES (64LL << 20)
/* Sharing contexts kept per resident dataset between jobs: a later job on the dataset reuses one
   instead of creating a context (allocations) and destroying it (cudaFree synchronises the whole
   device, so every job's teardown would wait for the other workers' kernels). */
#define SRV_IDLE_MAX 8

typedef struct srv_job {
  int64_t id;
  lagrbf_job_t spec;
  double *xd, *fd, *xp;   /* owned copies of the inputs */
  double *result;         /* np * dim positions */
  int state;              /* 0 queued, 1 running, 2 done, 3 collected */
  int rc;
  char err[256];
  double t_submit, t_start, t_done;
  double pss;             /* particle-steps advanced */
  struct srv_job *next;   /* FIFO */
} srv_job;

typedef struct {
  int64_t id;             /* > 0 */
  void *ctx;              /* the owner context (holds the dataset)                           */
  int busy;               /* the owner context runs a job                                    */
  int ready;              /* every patch set up and solved: other jobs may share the dataset */
  int users;              /* running jobs on the dataset (owner and sharing contexts)        */
  long long bytes;        /* estimate held by the owner context and the idle sharing contexts */
  int np_cap;
  double last_used;
  void *idle[SRV_IDLE_MAX];            /* idle contexts sharing this dataset, ready for reuse */
  long long idle_bytes[SRV_IDLE_MAX];  /* the device-memory estimate each of them holds    */
  int nidle;
} srv_dataset;

typedef struct {
  pthread_mutex_t lock, create_lock;
  pthread_cond_t cv_work, cv_done;
  srv_job *head, *tail;
  srv_job **jobs;
  int64_t njobs, capjobs;
  srv_dataset *ds;
  int nds, capds;
  long long budget, in_use;
  int nworkers, stop;
  pthread_t *threads;
  /* statistics since the last reset: latency, queue wait and service time of completed jobs */
  double *lat, *qwait, *svc;
  int64_t nlat, caplat, failed;
  double pss, t0, t_last;
} srv_t;

static double now_s(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* Device bytes of a particle swarm of np points and of a dataset of nd points (data arrays, patch
   coefficients, record blocks, factorisation workspace), deliberately generous. */
static long long pbytes(long long np, int dim)
{
  return np * (long long)(8 * dim * 12 + 64) + (16LL << 20);
}
static long long particle_bytes(const lagrbf_job_t *j) { return pbytes(j->np, j->dim); }
static long long dataset_bytes(const lagrbf_job_t *j)
{
  long long ncells = 1, nnodes = 1, m;
  int d;
  for (d = 0; d < j->dim; d++) {
    ncells *= (j->nodes[d] > 1 ? j->nodes[d] - 1 : 1);
    nnodes *= j->nodes[d];
  }
  m = 2LL * (1 << j->dim) * ((long long)j->nd / (ncells > 0 ? ncells : 1) + 1) + 16; /* largest patch, generous */
  {
    /* factorisation workspace: (1024 / LGB_FACT_T) patch slots per SM (160 SMs assumed), at most
       4 GB, as the context sizes it */
    long long ws = (1024LL / LGB_FACT_T) * 160 * m * m * 8;
    if (ws > (4LL << 30)) ws = 4LL << 30;
    return (long long)j->nd * (long long)(400 + 120 * (1 << j->dim) * j->dim) + nnodes * 64 + ws + (64LL << 20);
  }
}

static srv_dataset *find_ds(srv_t *s, int64_t id)
{
  int i;
  if (id <= 0) return NULL;
  for (i = 0; i < s->nds; i++)
    if (s->ds[i].id == id) return &s->ds[i];
  return NULL;
}

static void drop_ds(srv_t *s, int i)
{
  int k;
  for (k = 0; k < s->ds[i].nidle; k++) lagrbf_destroy(s->ds[i].idle[k]); /* they borrow the owner's arrays */
  if (s->ds[i].ctx) lagrbf_destroy(s->ds[i].ctx);
  s->in_use -= s->ds[i].bytes;
  s->ds[i] = s->ds[--s->nds];
}

/* Bytes a job adds to what is in use, given what is resident. */
static long long job_extra(srv_t *s, const srv_job *j)
{
  srv_dataset *d = find_ds(s, j->spec.dataset_id);
  if (d && d->busy) { /* a context sharing the dataset: an idle one is reused, growing if needed */
    const long long need = particle_bytes(&j->spec) + SHARE_BYTES;
    const long long held = d->nidle > 0 ? d->idle_bytes[d->nidle - 1] : 0;
    return need > held ? need - held : 0;
  }
  if (d) return (j->spec.np > d->np_cap) ? pbytes(j->spec.np, j->spec.dim) - pbytes(d->np_cap, j->spec.dim) : 0;
  return dataset_bytes(&j->spec) + particle_bytes(&j->spec);
}

/* A resident dataset may be evicted when idle, not the one wanted, and no queued job relies on it
   (a queued job without its own copy of the data). */
static int evictable(srv_t *s, const srv_dataset *d, int64_t keep)
{
  const srv_job *q;
  if (d->busy || d->users || d->id == keep) return 0;
  for (q = s->head; q; q = q->next)
    if (q->spec.dataset_id == d->id && !q->xd) return 0;
  return 1;
}

/* Makes room for `need` bytes by evicting idle resident datasets (least recently used first),
   keeping `keep`; evicts nothing and returns 0 when even evicting all candidates would not do. */
static int make_room(srv_t *s, long long need, int64_t keep)
{
  long long freeable = 0;
  int i;
  if (s->in_use + need <= s->budget) return 1;
  for (i = 0; i < s->nds; i++)
    if (evictable(s, &s->ds[i], keep)) freeable += s->ds[i].bytes;
  if (s->in_use - freeable + need > s->budget) return 0;
  while (s->in_use + need > s->budget) {
    int victim = -1;
    for (i = 0; i < s->nds; i++)
      if (evictable(s, &s->ds[i], keep) && (victim < 0 || s->ds[i].last_used < s->ds[victim].last_used)) victim = i;
    if (victim < 0) return 0;
    drop_ds(s, victim);
  }
  return 1;
}

/* First admissible job in FIFO order; jobs behind the head may pass it unless it has waited
   more than two seconds (so a large job is not starved). */
static srv_job *pick(srv_t *s)
{
  srv_job *j, *prev = NULL;
  double t = now_s();
  for (j = s->head; j; prev = j, j = j->next) {
    srv_dataset *d = find_ds(s, j->spec.dataset_id);
    int ok = !(d && d->busy && !d->ready); /* a busy dataset is shared once it is ready */
    if (ok && j->spec.dataset_id > 0 && !d && !j->xd) ok = 0; /* waits for its dataset to be resident */
    if (ok) ok = make_room(s, job_extra(s, j), j->spec.dataset_id);
    if (ok) {
      if (prev) prev->next = j->next;
      else s->head = j->next;
      if (s->tail == j) s->tail = prev;
      j->next = NULL;
      return j;
    }
    if (j == s->head && t - j->t_submit > 2.0) break;
  }
  return NULL;
}

static void *create_job_ctx(srv_t *s, const lagrbf_job_t *j)
{
  char v[256];
  void *ctx;
  int d;
  pthread_mutex_lock(&s->create_lock);
  lagrbf_options_clear();
  snprintf(v, sizeof(v), "%d", j->dim); lagrbf_options_set_value("pu_mesh_dim", v);
  v[0] = 0;
  for (d = 0; d < j->dim; d++) snprintf(v + strlen(v), sizeof(v) - strlen(v), d ? ",%d" : "%d", j->nodes[d]);
  lagrbf_options_set_value("pu_mesh_n", v);
  v[0] = 0;
  for (d = 0; d < j->dim; d++) snprintf(v + strlen(v), sizeof(v) - strlen(v), d ? ",%.17g" : "%.17g", j->O[d]);
  lagrbf_options_set_value("pu_mesh_O", v);
  v[0] = 0;
  for (d = 0; d < j->dim; d++) snprintf(v + strlen(v), sizeof(v) - strlen(v), d ? ",%.17g" : "%.17g", j->L[d]);
  lagrbf_options_set_value("pu_mesh_L", v);
  snprintf(v, sizeof(v), "%.17g", j->overlap); lagrbf_options_set_value("pu_mesh_overlap", v);
  snprintf(v, sizeof(v), "%.17g", j->shape_factor); lagrbf_options_set_value("pu_mesh_shape_factor", v);
  snprintf(v, sizeof(v), "%d", j->kernel); lagrbf_options_set_value("kernel_type", v);
  snprintf(v, sizeof(v), "%d", j->nfields); lagrbf_options_set_value("n_interpolation_fields", v);
  lagrbf_options_set_value("advection", "true");
  snprintf(v, sizeof(v), "%d", j->scheme); lagrbf_options_set_value("advection_scheme", v);
  snprintf(v, sizeof(v), "%.17g", j->dt); lagrbf_options_set_value("dt", v);
  snprintf(v, sizeof(v), "%.17g", j->cfl > 0 ? j->cfl : 0.3); lagrbf_options_set_value("cfl_fac", v);
  lagrbf_options_set_value("solve_method", "2");
  /* resident datasets set up every patch, so that later jobs can share them read-only */
  if (j->dataset_id > 0) lagrbf_options_set_value("setup_all_patches", "true");
  lagrbf_options_set_value("eval_precision", j->fp32 ? "fp32" : "fp64");
  ctx = lagrbf_create();
  if (!ctx) snprintf(v, sizeof(v), "%s", lagrbf_gpu_last_error());
  lagrbf_options_clear();
  pthread_mutex_unlock(&s->create_lock);
  if (!ctx) lgb_set_error_msg(LAGRBF_ERR_GPU, v);
  return ctx;
}

static void mark_ready(srv_t *s, int64_t id)
{
  srv_dataset *d;
  pthread_mutex_lock(&s->lock);
  d = find_ds(s, id);
  if (d && d->ctx && !d->ready) {
    d->ready = 1;
    pthread_cond_broadcast(&s->cv_work);
  }
  pthread_mutex_unlock(&s->lock);
}

/* Runs one job on ctx (the dataset is filled when `fill` is set; an owner context of a resident
   dataset marks it ready for sharing once its interpolation has set up every patch). */
static int run_job(srv_t *s, void *ctx, srv_job *j, int fill, int owner)
{
  const lagrbf_job_t *p = &j->spec;
  lagrbf_stats_t st0, st1;
  int64_t *pid = NULL;
  int rc = 0, k;
  double t = 0.0;
  if (fill && (rc = lagrbf_fill_swarm(ctx, true, p->nd, j->xd, j->fd, NULL))) return rc;
  if ((rc = lgb_ctx_set_scheme(ctx, p->scheme, p->dt, p->cfl > 0 ? p->cfl : 0.3))) return rc;
  if ((rc = lagrbf_gpu_set_precision(ctx, p->fp32))) return rc;
  pid = (int64_t *)malloc(sizeof(int64_t) * (size_t)(p->np > 0 ? p->np : 1));
  if (!pid) return lgb_set_error_msg(LAGRBF_ERR_MEM, "out of host memory");
  for (k = 0; k < p->np; k++) pid[k] = k + 1;
  rc = lagrbf_fill_swarm(ctx, false, p->np, j->xp, NULL, pid);
  free(pid);
  if (rc) return rc;
  if ((rc = lagrbf_interpolation(ctx))) return rc;
  if (owner && p->dataset_id > 0) mark_ready(s, p->dataset_id);
  if ((rc = lagrbf_gpu_get_stats(ctx, &st0))) return rc;
  for (k = 0; k < p->nsteps && !rc; k++, t += p->dt) rc = lagrbf_gpu_advect_resident(ctx, t, t + p->dt);
  if (rc) return rc;
  if ((rc = lagrbf_gpu_get_stats(ctx, &st1))) return rc;
  j->pss = (double)(st1.particle_steps - st0.particle_steps);
  return lagrbf_output(ctx, false, p->np, j->result, NULL, NULL, "fields");
}

static void *worker(void *arg)
{
  srv_t *s = (srv_t *)arg;
  pthread_mutex_lock(&s->lock);
  for (;;) {
    srv_job *j = NULL;
    srv_dataset *d;
    void *ctx = NULL, *share = NULL, *reuse = NULL;
    int fill = 0, cached, rc, owner = 0;
    long long extra, ctx_bytes;
    while (!s->stop && !(j = pick(s))) pthread_cond_wait(&s->cv_work, &s->lock);
    if (!j) break;
    j->state = 1;
    j->t_start = now_s();
    extra = job_extra(s, j);
    s->in_use += extra;
    ctx_bytes = extra;
    d = find_ds(s, j->spec.dataset_id);
    cached = j->spec.dataset_id > 0;
    if (d && d->busy) {
      /* the owner context is running: share its dataset from a context of this job (an idle one
         left by an earlier job if there is one; its bytes move from the dataset to this job) */
      d->users++;
      share = d->ctx;
      if (d->nidle > 0) {
        d->nidle--;
        reuse = d->idle[d->nidle];
        ctx_bytes += d->idle_bytes[d->nidle];
        d->bytes -= d->idle_bytes[d->nidle];
      }
    } else if (d) {
      d->busy = 1;
      d->users++;
      d->bytes += extra;
      if (j->spec.np > d->np_cap) d->np_cap = j->spec.np;
      ctx = d->ctx;
      owner = 1;
    } else if (cached) {
      if (s->nds == s->capds) {
        int cap = s->capds ? 2 * s->capds : 16;
        srv_dataset *nd = (srv_dataset *)realloc(s->ds, sizeof(srv_dataset) * (size_t)cap);
        if (nd) { s->ds = nd; s->capds = cap; }
      }
      if (s->nds == s->capds) cached = 0; /* no room in the table: run it as a private dataset */
    }
    if (!d && cached) {
      d = &s->ds[s->nds++];
      memset(d, 0, sizeof(*d));
      d->id = j->spec.dataset_id;
      d->busy = 1;
      d->users = 1;
      d->bytes = extra;
      d->np_cap = j->spec.np;
      owner = 1;
    }
    pthread_mutex_unlock(&s->lock);

    rc = 0;
    if (reuse) {
      ctx = reuse; /* already shares this dataset */
    } else if (share) {
      ctx = create_job_ctx(s, &j->spec);
      rc = ctx ? lagrbf_gpu_share_dataset(ctx, share) : LAGRBF_ERR_GPU;
    } else if (!ctx) {
      ctx = create_job_ctx(s, &j->spec);
      fill = 1;
      if (!ctx) rc = LAGRBF_ERR_GPU;
      if (ctx && owner) { /* the dataset's owner context, known before it is marked ready */
        pthread_mutex_lock(&s->lock);
        d = find_ds(s, j->spec.dataset_id);
        if (d && !d->ctx) d->ctx = ctx;
        pthread_mutex_unlock(&s->lock);
      }
    }
    if (!rc) rc = run_job(s, ctx, j, fill, owner);
    if (rc) snprintf(j->err, sizeof(j->err), "%s", lagrbf_gpu_last_error());

    pthread_mutex_lock(&s->lock);
    d = find_ds(s, j->spec.dataset_id);
    if (d && owner && d->busy && (!d->ctx || d->ctx == ctx)) {
      d->ctx = ctx;
      d->busy = 0;
      d->users--;
      d->last_used = now_s();
      if (rc && d->users == 0) drop_ds(s, (int)(d - s->ds)); /* a failed context is not reused */
      else if (rc) d->ready = 0;
    } else if (d && share && ctx && !rc && !s->stop && d->nidle < SRV_IDLE_MAX) {
      /* keep the sharing context for the next job on this dataset; its bytes stay in use, held by
         the dataset (an eviction frees them with it) */
      d->idle[d->nidle] = ctx;
      d->idle_bytes[d->nidle] = ctx_bytes;
      d->nidle++;
      d->bytes += ctx_bytes;
      d->users--;
      d->last_used = now_s();
    } else {
      if (ctx) lagrbf_destroy(ctx);
      s->in_use -= ctx_bytes;
      if (d && share) {
        d->users--;
        d->last_used = now_s();
      }
    }
    j->rc = rc;
    j->t_done = now_s();
    j->state = 2;
    free(j->xd); free(j->fd); free(j->xp);
    j->xd = j->fd = j->xp = NULL;
    if (rc) s->failed++;
    else {
      if (s->nlat == s->caplat) {
        int64_t cap = s->caplat ? 2 * s->caplat : 1024;
        double *nl = (double *)realloc(s->lat, sizeof(double) * (size_t)cap);
        double *nq = (double *)realloc(s->qwait, sizeof(double) * (size_t)cap);
        double *ns = (double *)realloc(s->svc, sizeof(double) * (size_t)cap);
        if (nl) s->lat = nl;
        if (nq) s->qwait = nq;
        if (ns) s->svc = ns;
        if (nl && nq && ns) s->caplat = cap;
      }
      if (s->nlat < s->caplat) {
        s->lat[s->nlat] = 1e3 * (j->t_done - j->t_submit);
        s->qwait[s->nlat] = 1e3 * (j->t_start - j->t_submit);
        s->svc[s->nlat] = 1e3 * (j->t_done - j->t_start);
        s->nlat++;
      }
      s->pss += j->pss;
      s->t_last = j->t_done;
    }
    pthread_cond_broadcast(&s->cv_done);
    pthread_cond_broadcast(&s->cv_work);
  }
  pthread_mutex_unlock(&s->lock);
  return NULL;
}

LAGRBF_EXPORT void *lagrbf_server_create(double hbm_budget_bytes, int32_t nworkers)
{
  srv_t *s;
  int i;
  if (!(hbm_budget_bytes > 0.0) || nworkers < 1 || nworkers > 256) {
    lgb_set_error_msg(LAGRBF_ERR_ARG_OUTOFRANGE, "server: budget must be positive and workers in [1, 256]");
    return NULL;
  }
  s = (srv_t *)calloc(1, sizeof(srv_t));
  if (!s) return NULL;
  pthread_mutex_init(&s->lock, NULL);
  pthread_mutex_init(&s->create_lock, NULL);
  pthread_cond_init(&s->cv_work, NULL);
  pthread_cond_init(&s->cv_done, NULL);
  s->budget = (long long)hbm_budget_bytes;
  s->nworkers = nworkers;
  s->t0 = now_s();
  s->threads = (pthread_t *)calloc((size_t)nworkers, sizeof(pthread_t));
  for (i = 0; i < nworkers; i++) pthread_create(&s->threads[i], NULL, worker, s);
  return s;
}

static double *dup_array(const double *a, size_t n)
{
  double *b = (double *)malloc(sizeof(double) * (n ? n : 1));
  if (b && a && n) memcpy(b, a, sizeof(double) * n);
  return b;
}

LAGRBF_EXPORT int lagrbf_server_submit(void *srv, const lagrbf_job_t *job, int64_t *job_id)
{
  srv_t *s = (srv_t *)srv;
  srv_job *j;
  if (!s || !job || !job_id) return lgb_set_error_msg(LAGRBF_ERR_ARG_NULL, "server: NULL argument");
  if ((job->dim != 2 && job->dim != 3) || job->np < 0 || job->nsteps < 0 || job->nd < 0 || job->nfields < job->dim ||
      job->scheme < 0 || job->scheme > 3 || !(job->dt > 0.0))
    return lgb_set_error_msg(LAGRBF_ERR_ARG_OUTOFRANGE, "server: invalid job description");
  if (job->np > 0 && !job->particles) return lgb_set_error_msg(LAGRBF_ERR_ARG_NULL, "server: NULL particles");
  if (job->dataset_id <= 0 && (!job->data_coords || !job->data_values))
    return lgb_set_error_msg(LAGRBF_ERR_ARG_NULL, "server: a job without a dataset id needs its data");
  if (dataset_bytes(job) + particle_bytes(job) > s->budget)
    return lgb_set_error_msg(LAGRBF_ERR_MEM, "server: the job alone exceeds the device-memory budget");
  if (job->dataset_id > 0 && !(job->data_coords && job->data_values)) {
    /* the dataset must be resident, or come with a job already queued or running */
    int known;
    int64_t k;
    pthread_mutex_lock(&s->lock);
    known = find_ds(s, job->dataset_id) != NULL;
    for (k = 0; k < s->njobs && !known; k++)
      known = s->jobs[k]->state < 2 && s->jobs[k]->spec.dataset_id == job->dataset_id && s->jobs[k]->xd;
    pthread_mutex_unlock(&s->lock);
    if (!known) return lgb_set_error_msg(LAGRBF_ERR_ARG_WRONGSTATE, "server: unknown dataset id and no data given");
  }
  j = (srv_job *)calloc(1, sizeof(srv_job));
  if (!j) return lgb_set_error_msg(LAGRBF_ERR_MEM, "out of host memory");
  j->spec = *job;
  if (job->data_coords && job->data_values) {
    j->xd = dup_array(job->data_coords, (size_t)job->nd * job->dim);
    j->fd = dup_array(job->data_values, (size_t)job->nd * job->nfields);
  }
  j->xp = dup_array(job->particles, (size_t)job->np * job->dim);
  j->result = (double *)calloc((size_t)(job->np > 0 ? job->np : 1) * job->dim, sizeof(double));
  j->spec.data_coords = j->spec.data_values = j->spec.particles = NULL;
  if (!j->xp || !j->result || ((job->data_coords && job->data_values) && (!j->xd || !j->fd))) {
    free(j->xd); free(j->fd); free(j->xp); free(j->result); free(j);
    return lgb_set_error_msg(LAGRBF_ERR_MEM, "out of host memory");
  }
  pthread_mutex_lock(&s->lock);
  if (s->njobs == s->capjobs) {
    int64_t cap = s->capjobs ? 2 * s->capjobs : 1024;
    srv_job **nj = (srv_job **)realloc(s->jobs, sizeof(srv_job *) * (size_t)cap);
    if (!nj) {
      pthread_mutex_unlock(&s->lock);
      free(j->xd); free(j->fd); free(j->xp); free(j->result); free(j);
      return lgb_set_error_msg(LAGRBF_ERR_MEM, "out of host memory");
    }
    s->jobs = nj;
    s->capjobs = cap;
  }
  s->jobs[s->njobs] = j;
  j->id = ++s->njobs;
  j->t_submit = now_s();
  if (s->tail) s->tail->next = j;
  else s->head = j;
  s->tail = j;
  *job_id = j->id;
  pthread_cond_broadcast(&s->cv_work);
  pthread_mutex_unlock(&s->lock);
  return 0;
}

LAGRBF_EXPORT int lagrbf_server_wait(void *srv, int64_t job_id, double *positions, double *latency_ms)
{
  srv_t *s = (srv_t *)srv;
  srv_job *j;
  int rc;
  if (!s) return lgb_set_error_msg(LAGRBF_ERR_ARG_NULL, "server is NULL");
  pthread_mutex_lock(&s->lock);
  if (job_id < 1 || job_id > s->njobs) { pthread_mutex_unlock(&s->lock); return lgb_set_error_msg(LAGRBF_ERR_ARG_OUTOFRANGE, "server: unknown job"); }
  j = s->jobs[job_id - 1];
  while (j->state < 2) pthread_cond_wait(&s->cv_done, &s->lock);
  if (j->state == 3) { pthread_mutex_unlock(&s->lock); return lgb_set_error_msg(LAGRBF_ERR_ARG_WRONGSTATE, "server: job already collected"); }
  rc = j->rc;
  if (!rc && positions) memcpy(positions, j->result, sizeof(double) * (size_t)j->spec.np * j->spec.dim);
  if (latency_ms) *latency_ms = 1e3 * (j->t_done - j->t_submit);
  free(j->result);
  j->result = NULL;
  j->state = 3;
  pthread_mutex_unlock(&s->lock);
  if (rc) lgb_set_error_msg(rc, j->err);
  return rc;
}

static int cmp_d(const void *a, const void *b)
{
  double x = *(const double *)a, y = *(const double *)b;
  return (x > y) - (x < y);
}

LAGRBF_EXPORT int lagrbf_server_stats(void *srv, lagrbf_server_stats_t *st)
{
  srv_t *s = (srv_t *)srv;
  srv_job *j;
  int64_t i;
  if (!s || !st) return lgb_set_error_msg(LAGRBF_ERR_ARG_NULL, "server: NULL argument");
  memset(st, 0, sizeof(*st));
  pthread_mutex_lock(&s->lock);
  st->submitted = s->njobs;
  st->completed = s->nlat;
  st->failed = s->failed;
  for (j = s->head; j; j = j->next) st->queued++;
  for (i = 0; i < s->njobs; i++) st->running += (s->jobs[i]->state == 1);
  st->particle_steps = s->pss;
  st->elapsed_s = (s->t_last > s->t0 ? s->t_last : now_s()) - s->t0;
  st->datasets_resident = s->nds;
  st->bytes_in_use = (double)s->in_use;
  if (s->nlat > 0) {
    double *c = (double *)malloc(sizeof(double) * (size_t)s->nlat), sum = 0.0;
    if (c) {
      memcpy(c, s->lat, sizeof(double) * (size_t)s->nlat);
      qsort(c, (size_t)s->nlat, sizeof(double), cmp_d);
      for (i = 0; i < s->nlat; i++) sum += c[i];
      /* nearest-rank percentiles */
      st->p50_ms = c[(int64_t)ceil(0.50 * (double)s->nlat) - 1];
      st->p99_ms = c[(int64_t)ceil(0.99 * (double)s->nlat) - 1];
      st->mean_ms = sum / (double)s->nlat;
      st->max_ms = c[s->nlat - 1];
      memcpy(c, s->qwait, sizeof(double) * (size_t)s->nlat);
      qsort(c, (size_t)s->nlat, sizeof(double), cmp_d);
      st->queue_p50_ms = c[(int64_t)ceil(0.50 * (double)s->nlat) - 1];
      st->queue_p99_ms = c[(int64_t)ceil(0.99 * (double)s->nlat) - 1];
      memcpy(c, s->svc, sizeof(double) * (size_t)s->nlat);
      qsort(c, (size_t)s->nlat, sizeof(double), cmp_d);
      st->service_p50_ms = c[(int64_t)ceil(0.50 * (double)s->nlat) - 1];
      st->service_p99_ms = c[(int64_t)ceil(0.99 * (double)s->nlat) - 1];
      free(c);
    }
  }
  pthread_mutex_unlock(&s->lock);
  return 0;
}

LAGRBF_EXPORT int lagrbf_server_reset_stats(void *srv)
{
  srv_t *s = (srv_t *)srv;
  if (!s) return lgb_set_error_msg(LAGRBF_ERR_ARG_NULL, "server is NULL");
  pthread_mutex_lock(&s->lock);
  s->nlat = 0;
  s->failed = 0;
  s->pss = 0.0;
  s->t0 = now_s();
  s->t_last = 0.0;
  pthread_mutex_unlock(&s->lock);
  return 0;
}

LAGRBF_EXPORT void lagrbf_server_destroy(void *srv)
{
  srv_t *s = (srv_t *)srv;
  int i;
  int64_t k;
  if (!s) return;
  pthread_mutex_lock(&s->lock);
  /* queued jobs are cancelled; running jobs finish */
  while (s->head) {
    srv_job *j = s->head;
    s->head = j->next;
    j->rc = LAGRBF_ERR_ARG_WRONGSTATE;
    snprintf(j->err, sizeof(j->err), "server destroyed before the job ran");
    j->state = 2;
  }
  s->tail = NULL;
  s->stop = 1;
  pthread_cond_broadcast(&s->cv_work);
  pthread_cond_broadcast(&s->cv_done);
  pthread_mutex_unlock(&s->lock);
  for (i = 0; i < s->nworkers; i++) pthread_join(s->threads[i], NULL);
  while (s->nds > 0) drop_ds(s, s->nds - 1); /* sharing contexts before their owner */
  for (k = 0; k < s->njobs; k++) {
    srv_job *j = s->jobs[k];
    free(j->xd); free(j->fd); free(j->xp); free(j->result); free(j);
  }
  free(s->jobs); free(s->ds); free(s->lat); free(s->qwait); free(s->svc); free(s->threads);
  pthread_mutex_destroy(&s->lock);
  pthread_mutex_destroy(&s->create_lock);
  pthread_cond_destroy(&s->cv_work);
  pthread_cond_destroy(&s->cv_done);
  free(s);
}
