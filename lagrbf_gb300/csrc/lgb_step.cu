/*
 * lgb_step.cu -- explicit advection stages and the device-side step control.
 *
 * Replaces AdvectionExplicit_Scalar (src/advection/advection.c:36-57), the stage drivers of
 * runge_kutta_1.c:37-75, runge_kutta_2.c:38-91, runge_kutta_4.c:45-156 and dormand_prince.c:
 * 37-310, AdvectionComputeTimestep_CFL (advection.c:430-470), AdvectionCopyVelocityField
 * (advection.c:298-316) and the loop scalars of InternalForwardAdvectionLoop (time_loop.c:39-100).
 *
 * Every stage is one pass over the particles that writes the stage position (and commits the
 * previous stage velocity into v_adv), followed by re-binning and one evaluation.  The global
 * reductions of the reference (CFL min dt, DOPRI max error: MPI_Allreduce sites advection.c:466,
 * dormand_prince.c:93) are warp-reduced atomics on the ordered bit patterns of non-negative
 * doubles.  The loop scalars (t, dt, DOPRI dt) live in a device control block, so a whole
 * internal step is a fixed sequence of launches that the host captures once in a CUDA graph.
 */
#include <math.h>
#include "lgb_common.cuh"
#include <float.h>

__constant__ double c_dp_a[6][6] = {
  {1.0 / 5.0, 0, 0, 0, 0, 0},
  {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0},
  {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0},
  {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0},
  {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0},
  {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0}};
__constant__ double c_dp_e[7] = {5179.0 / 57600.0, 0, 7571.0 / 16695.0, 393.0 / 640.0, -92097.0 / 339200.0,
                                 187.0 / 2100.0, 1.0 / 40.0};

/* AdvectionProjectOntoSphereBoundary_Pointwise (advection.c:472-491) */
__device__ __forceinline__ void project_sphere(double *x, int dim, double rmin, double rmax)
{
  double pos = 0.0, normal[3];
  for (int d = 0; d < dim; d++) pos += x[d] * x[d];
  if (pos < rmax * rmax && pos > rmin * rmin) return;
  pos = sqrt(pos);
  for (int d = 0; d < dim; d++) normal[d] = x[d] / pos;
  if (pos > rmax) for (int d = 0; d < dim; d++) x[d] = rmax * normal[d];
  else for (int d = 0; d < dim; d++) x[d] = rmin * normal[d];
}

struct StageParams {
  int np, dim, scheme, stage;
  double *xp, *x0, *vel, *vadv;
  const int *alive;
  const lgb_ctrl *ctrl;
  const double *hcur;  /* per-particle Dormand-Prince: the particle's step (else NULL: ctrl->dt) */
  const int *active;   /* per-particle Dormand-Prince: particles taking part in the sweep      */
};

__global__ void k_stage(StageParams S)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= S.np || !S.alive[p]) return;
  if (S.active && !S.active[p]) return;
  const int dim = S.dim;
  const double dt = S.hcur ? S.hcur[p] : S.ctrl->dt;
  const double rmin = S.ctrl->rmin, rmax = S.ctrl->rmax;
  const size_t o = (size_t)p * dim;
  const size_t st = (size_t)S.np * dim; /* stride between v_adv stages */
  double x[3], x0[3], v[3];
  for (int d = 0; d < dim; d++) { x[d] = S.xp[o + d]; v[d] = S.vel[o + d]; }
  switch (S.scheme) {
  case LGB_RK1:
    /* runge_kutta_1.c:61-64: x = x0 + dt * v */
    for (int d = 0; d < dim; d++) S.xp[o + d] = x[d] + dt * v[d];
    return;
  case LGB_RK2:
    if (S.stage == 0) {
      for (int d = 0; d < dim; d++) { S.x0[o + d] = x[d]; S.xp[o + d] = x[d] + (0.5 * dt) * v[d]; }
    } else {
      for (int d = 0; d < dim; d++) S.xp[o + d] = S.x0[o + d] + dt * v[d];
    }
    return;
  case LGB_RK4: {
    const double c[3] = {0.5, 0.5, 1.0};
    if (S.stage == 0) for (int d = 0; d < dim; d++) x0[d] = x[d];
    else for (int d = 0; d < dim; d++) x0[d] = S.x0[o + d];
    /* commit v_adv_{stage} = velocity (stage 0: AdvectionSetInitialValues) */
    for (int d = 0; d < dim; d++) S.vadv[S.stage * st + o + d] = v[d];
    if (S.stage == 0) for (int d = 0; d < dim; d++) S.x0[o + d] = x0[d];
    if (S.stage < 3) {
      double xs[3];
      for (int d = 0; d < dim; d++) xs[d] = x0[d] + (c[S.stage] * dt) * v[d];
      project_sphere(xs, dim, rmin, rmax);
      for (int d = 0; d < dim; d++) S.xp[o + d] = xs[d];
    } else {
      const double w[4] = {1.0, 2.0, 2.0, 1.0};
      double xs[3];
      for (int d = 0; d < dim; d++) xs[d] = x[d]; /* components not yet updated keep the stage-3 value */
      for (int d = 0; d < dim; d++) {
        double sum = 0.0;
        for (int s = 0; s < 4; s++) sum += w[s] * S.vadv[s * st + o + d];
        xs[d] = x0[d] + dt / 6.0 * sum;
        project_sphere(xs, dim, rmin, rmax); /* runge_kutta_4.c:140, inside the component loop */
      }
      for (int d = 0; d < dim; d++) S.xp[o + d] = xs[d];
    }
    return;
  }
  case LGB_DOPRI: {
    const int s = S.stage; /* 0..5 */
    if (s == 0) for (int d = 0; d < dim; d++) { x0[d] = x[d]; S.x0[o + d] = x[d]; }
    else for (int d = 0; d < dim; d++) x0[d] = S.x0[o + d];
    for (int d = 0; d < dim; d++) S.vadv[s * st + o + d] = v[d];
    double vs[3] = {0.0, 0.0, 0.0}, xs[3];
    for (int j = 0; j <= s; j++)
      for (int d = 0; d < dim; d++) {
        double vj = (j == s) ? v[d] : S.vadv[j * st + o + d];
        vs[d] += c_dp_a[s][j] * vj;
      }
    for (int d = 0; d < dim; d++) { S.vel[o + d] = vs[d]; xs[d] = x0[d] + dt * vs[d]; }
    project_sphere(xs, dim, rmin, rmax);
    for (int d = 0; d < dim; d++) S.xp[o + d] = xs[d];
    return;
  }
  default: return;
  }
}

extern "C" int lgb_op_stage(lgb_dev *d, int scheme, int stage, void *stream)
{
  if (d->np <= 0) return 0;
  StageParams S;
  S.np = d->np; S.dim = d->g.dim; S.scheme = scheme; S.stage = stage;
  S.xp = d->xp; S.x0 = d->x0; S.vel = d->vel; S.vadv = d->vadv; S.alive = d->alive; S.ctrl = d->ctrl;
  const int pp = (scheme == LGB_DOPRI && d->dopri_pp);
  S.hcur = pp ? d->hcur : NULL;
  S.active = pp ? d->active : NULL;
  k_stage<<<lgb_cdiv(d->np, 256), 256, 0, (cudaStream_t)stream>>>(S);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}

/* DOPRI embedded error (dormand_prince.c:37-102): commits v_adv_6, per-particle error norm,
   global max. */
__global__ void k_dopri_error(int np, int dim, const double *__restrict__ xp, const double *__restrict__ x0,
                              const double *__restrict__ vel, double *__restrict__ vadv,
                              const int *__restrict__ alive, lgb_ctrl *ctrl)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  double E = -1.0;
  if (p < np && alive[p]) {
    const size_t o = (size_t)p * dim, st = (size_t)np * dim;
    const double dt = ctrl->dt, atol = ctrl->dopri_atol, rtol = ctrl->dopri_rtol;
    for (int d = 0; d < dim; d++) vadv[6 * st + o + d] = vel[o + d];
    double vlow[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 7; i++)
      for (int d = 0; d < dim; d++) vlow[d] += c_dp_e[i] * vadv[i * st + o + d];
    double e2 = 0.0;
    for (int d = 0; d < dim; d++) {
      double xa = x0[o + d], xb = xp[o + d];
      double mv = (fabs(xa) < fabs(xb)) ? fabs(xb) : fabs(xa);
      double tol = atol + rtol * mv;
      double err = xb - (xa + dt * vlow[d]);
      e2 += (err * err) / (tol * tol);
    }
    E = sqrt(1.0 / dim * e2);
  }
  /* block max then one atomic per block (E >= 0 orders like its bit pattern) */
  __shared__ double s_e[32];
  for (int off = 16; off > 0; off >>= 1) E = fmax(E, __shfl_down_sync(0xffffffffu, E, off));
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) s_e[warp] = E;
  __syncthreads();
  if (warp == 0) {
    E = (lane < nw) ? s_e[lane] : -1.0;
    for (int off = 16; off > 0; off >>= 1) E = fmax(E, __shfl_down_sync(0xffffffffu, E, off));
    if (lane == 0 && E >= 0.0) {
      atomicMax(&ctrl->maxerr_bits, (unsigned long long)__double_as_longlong(E));
      ctrl->any_alive = 1;
    }
  }
}

extern "C" int lgb_op_dopri_error(lgb_dev *d, void *stream)
{
  if (d->np <= 0) return 0;
  k_dopri_error<<<lgb_cdiv(d->np, 256), 256, 0, (cudaStream_t)stream>>>(d->np, d->g.dim, d->xp, d->x0, d->vel,
                                                                          d->vadv, d->alive, d->ctrl);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}

/* ---- per-particle adaptive Dormand-Prince (an extension: the reference's scheme takes one global
   step from the global maximum error and always accepts it, dormand_prince.c:93,179-214).  Every
   live particle short of t_next attempts h_p = min(hp_p, its own CFL step cfl r / (|v_p| + 1e-16),
   t_next - tp_p) through the same six stages; the stage evaluations see only those particles.  The
   error norm E_p is the reference's (dormand_prince.c:68-91) for that particle; E_p <= 1 (or
   h_p < hmin, so that no particle stalls) accepts the step, else the particle returns to x0; either
   way hp_p = h_p min(fac_max', max(fac_min, fac E_p^-1/5)), fac_max' = fac_max after an accepted
   step and 1 after a rejected one. ---- */
__global__ void k_pp_init(int np, const int *__restrict__ alive, double *__restrict__ tp, double *__restrict__ hp,
                          double t, const lgb_ctrl *ctrl)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  tp[p] = t;
  if (!(hp[p] > 0.0)) hp[p] = ctrl->dt_adv;
}

__global__ void k_pp_begin(int np, int dim, const int *__restrict__ alive, const double *__restrict__ vel,
                           const double *__restrict__ tp, const double *__restrict__ hp, double *__restrict__ hcur,
                           int *__restrict__ active, const lgb_ctrl *ctrl)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const double t_next = ctrl->t_next;
  const int act = alive[p] && tp[p] < t_next;
  active[p] = act;
  double h = 0.0;
  if (act) {
    double n2 = 0.0;
    for (int d = 0; d < dim; d++) n2 += vel[(size_t)p * dim + d] * vel[(size_t)p * dim + d];
    const double cfl = ctrl->cfl_fac * ctrl->cfl_radius / (sqrt(n2) + 1e-16);
    h = (hp[p] < cfl) ? hp[p] : cfl;
    if (tp[p] + h >= t_next) h = -(t_next - tp[p]); /* negative: clamped to t_next */
  }
  hcur[p] = h;
}

/* The stages read |hcur|; the sign marks a step clamped to t_next. */
__global__ void k_pp_abs(int np, double *__restrict__ hcur, double *__restrict__ hsign)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  const double h = hcur[p];
  hsign[p] = h;
  hcur[p] = fabs(h);
}

__global__ void k_pp_accept(int np, int dim, double *__restrict__ xp, const double *__restrict__ x0,
                            const double *__restrict__ vel, double *__restrict__ vadv, const int *__restrict__ alive,
                            const int *__restrict__ active, double *__restrict__ tp, double *__restrict__ hp,
                            const double *__restrict__ hsign, lgb_ctrl *ctrl)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  int acc = 0, left = 0;
  if (p < np && alive[p] && active[p]) {
    const size_t o = (size_t)p * dim, st = (size_t)np * dim;
    const double hs = hsign[p], h = fabs(hs), atol = ctrl->dopri_atol, rtol = ctrl->dopri_rtol;
    for (int d = 0; d < dim; d++) vadv[6 * st + o + d] = vel[o + d];
    double vlow[3] = {0.0, 0.0, 0.0};
    for (int i = 0; i < 7; i++)
      for (int d = 0; d < dim; d++) vlow[d] += c_dp_e[i] * vadv[i * st + o + d];
    double e2 = 0.0;
    for (int d = 0; d < dim; d++) {
      const double xa = x0[o + d], xb = xp[o + d];
      const double mv = (fabs(xa) < fabs(xb)) ? fabs(xb) : fabs(xa);
      const double tol = atol + rtol * mv;
      const double err = xb - (xa + h * vlow[d]);
      e2 += (err * err) / (tol * tol);
    }
    const double E = sqrt(1.0 / dim * e2);
    acc = (E <= 1.0) || (h < ctrl->pp_hmin);
    if (acc) {
      tp[p] = (hs < 0.0) ? ctrl->t_next : tp[p] + h;
    } else {
      for (int d = 0; d < dim; d++) xp[o + d] = x0[o + d];
    }
    const double fmx = (E <= 1.0) ? ctrl->dopri_fac_max : 1.0;
    const double q = ctrl->dopri_fac * pow(1.0 / E, 1.0 / 5.0);
    const double inner = (ctrl->dopri_fac_min < q) ? q : ctrl->dopri_fac_min;
    hp[p] = h * ((fmx < inner) ? fmx : inner);
    left = tp[p] < ctrl->t_next;
  } else if (p < np && alive[p]) {
    left = tp[p] < ctrl->t_next;
  }
  /* block sums, then one atomic each per block */
  __shared__ int s_a[32], s_l[32];
  for (int off = 16; off > 0; off >>= 1) {
    acc += __shfl_down_sync(0xffffffffu, acc, off);
    left += __shfl_down_sync(0xffffffffu, left, off);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) { s_a[warp] = acc; s_l[warp] = left; }
  __syncthreads();
  if (warp == 0) {
    acc = (lane < nw) ? s_a[lane] : 0;
    left = (lane < nw) ? s_l[lane] : 0;
    for (int off = 16; off > 0; off >>= 1) {
      acc += __shfl_down_sync(0xffffffffu, acc, off);
      left += __shfl_down_sync(0xffffffffu, left, off);
    }
    if (lane == 0) {
      if (acc) atomicAdd((unsigned long long *)&ctrl->particle_steps, (unsigned long long)acc);
      if (left) atomicAdd(&ctrl->pp_left, left);
    }
  }
}

extern "C" int lgb_op_pp_init(lgb_dev *d, double t, void *stream)
{
  if (d->np <= 0) return 0;
  k_pp_init<<<lgb_cdiv(d->np, 256), 256, 0, (cudaStream_t)stream>>>(d->np, d->alive, d->tp, d->hp, t, d->ctrl);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}

extern "C" int lgb_op_pp_begin(lgb_dev *d, void *stream)
{
  if (d->np <= 0) return 0;
  cudaStream_t s = (cudaStream_t)stream;
  /* hcur has 2 np entries: the stages read |h| from the first half, the acceptance the signed step
     (negative: clamped to t_next) from the second */
  k_pp_begin<<<lgb_cdiv(d->np, 256), 256, 0, s>>>(d->np, d->g.dim, d->alive, d->vel, d->tp, d->hp, d->hcur, d->active,
                                                 d->ctrl);
  k_pp_abs<<<lgb_cdiv(d->np, 256), 256, 0, s>>>(d->np, d->hcur, d->hcur + d->np);
  lgb_count_launch(2);
  return (int)cudaGetLastError();
}

extern "C" int lgb_op_pp_accept(lgb_dev *d, void *stream)
{
  if (d->np <= 0) return 0;
  k_pp_accept<<<lgb_cdiv(d->np, 256), 256, 0, (cudaStream_t)stream>>>(
      d->np, d->g.dim, d->xp, d->x0, d->vel, d->vadv, d->alive, d->active, d->tp, d->hp, d->hcur + d->np, d->ctrl);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}

/* velocity <- fields[:, :dim] (when copy), then CFL dt = min cfl*radius/(|v| + 1e-16) and the
   number of live particles. */
/* AdvectionComputeTimestep_CFL (advection.c:430-470): dt = min_p cfl * r / (|v_p| + 1e-16).  Every
   step of that expression is a correctly rounded monotone function of |v_p|^2 (sqrt and + rise,
   the division falls), so the minimum over particles is the expression at the largest |v_p|^2,
   bit for bit: the kernel only reduces max |v_p|^2 (one FMA chain per particle instead of a square
   root and a division on the FP64 pipe), and k_ctrl evaluates the expression once. */
__global__ void k_velocity_cfl(int np, int dim, int F, int copy, const double *__restrict__ fields,
                               double *__restrict__ vel, const int *__restrict__ alive, lgb_ctrl *ctrl)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned long long nb = 0ull; /* 1 + bits of |v|^2, 0: none (NaN speeds are skipped, as fmin does) */
  int live = 0;
  if (p < np && alive[p]) {
    live = 1;
    double n2 = 0.0;
    for (int d = 0; d < dim; d++) {
      double v = copy ? ((d < F) ? fields[(size_t)p * F + d] : 0.0) : vel[(size_t)p * dim + d];
      if (copy) vel[(size_t)p * dim + d] = v;
      n2 += v * v;
    }
    if (n2 == n2) nb = (unsigned long long)__double_as_longlong(n2) + 1ull;
  }
  /* block reduction, then one atomic per block: per-warp atomics on these two words serialise */
  __shared__ unsigned long long s_nb[32];
  __shared__ int s_live[32];
  for (int off = 16; off > 0; off >>= 1) {
    const unsigned long long o = __shfl_down_sync(0xffffffffu, nb, off);
    nb = (o > nb) ? o : nb;
    live += __shfl_down_sync(0xffffffffu, live, off);
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
  if (lane == 0) { s_nb[warp] = nb; s_live[warp] = live; }
  __syncthreads();
  if (warp == 0) {
    nb = (lane < nw) ? s_nb[lane] : 0ull;
    live = (lane < nw) ? s_live[lane] : 0;
    for (int off = 16; off > 0; off >>= 1) {
      const unsigned long long o = __shfl_down_sync(0xffffffffu, nb, off);
      nb = (o > nb) ? o : nb;
      live += __shfl_down_sync(0xffffffffu, live, off);
    }
    if (lane == 0) {
      if (nb) atomicMax(&ctrl->n2max_bits, nb);
      if (live) atomicAdd(&ctrl->np_alive, live);
    }
  }
}

extern "C" int lgb_op_copy_velocity(lgb_dev *d, void *stream)
{
  if (d->np <= 0) return 0;
  k_velocity_cfl<<<lgb_cdiv(d->np, 256), 256, 0, (cudaStream_t)stream>>>(d->np, d->g.dim, d->F, 1, d->fields,
                                                                           d->vel, d->alive, d->ctrl);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}

extern "C" int lgb_op_count_alive(lgb_dev *d, void *stream)
{
  if (d->np <= 0) return 0;
  k_velocity_cfl<<<lgb_cdiv(d->np, 256), 256, 0, (cudaStream_t)stream>>>(d->np, d->g.dim, d->F, 0, d->fields,
                                                                           d->vel, d->alive, d->ctrl);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}

/* Analytical velocity evaluated on the device at the live particles, in place of the host
   callback of AdvectionEvaluateVelocityFunction (advection.c:318-351), so that analytical advection
   needs no host round trip per stage.  Fields (par = parameters):
     ROTATION  par {omega, cx, cy}: v = omega (-(y - cy), x - cx, 0)
     CELLULAR  par {a, k}:          v = a (sin(k pi x) cos(k pi y), -cos(k pi x) sin(k pi y), 0)
     ABC       par {A, B, C, s}:    X = s x: v = (A sin Z + C cos Y, B sin X + A cos Z, C sin Y + B cos X)
     FOURIER   par {n, then n x (k1, k2, k3, phase, a1, a2, a3)}:
                                    v_c = sum_m a_mc sin(2 pi (k_m . x) + phase_m)
   Velocities of removed particles are left as they are, like the host path. */
__global__ void k_velocity_field(int np, int dim, const double *__restrict__ x, const int *__restrict__ alive,
                                 double *__restrict__ v, int kind, const double *__restrict__ par, int npar)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np || !alive[p]) return;
  const double *xp = x + (size_t)p * dim;
  double X = xp[0], Y = xp[1], Z = (dim == 3) ? xp[2] : 0.0;
  double o[3] = {0.0, 0.0, 0.0};
  switch (kind) {
  case LGB_VF_ROTATION:
    o[0] = -par[0] * (Y - par[2]);
    o[1] = par[0] * (X - par[1]);
    break;
  case LGB_VF_CELLULAR: {
    const double kx = par[1] * M_PI * X, ky = par[1] * M_PI * Y;
    o[0] = par[0] * sin(kx) * cos(ky);
    o[1] = -par[0] * cos(kx) * sin(ky);
    break;
  }
  case LGB_VF_ABC: {
    const double a = par[3] * X, b = par[3] * Y, c = par[3] * Z;
    o[0] = par[0] * sin(c) + par[2] * cos(b);
    o[1] = par[1] * sin(a) + par[0] * cos(c);
    o[2] = par[2] * sin(b) + par[1] * cos(a);
    break;
  }
  case LGB_VF_FOURIER: {
    const int nm = (int)par[0];
    for (int m = 0; m < nm && 1 + 7 * m + 6 < npar; m++) {
      const double *q = par + 1 + 7 * m;
      const double s = sin(2.0 * M_PI * (q[0] * X + q[1] * Y + q[2] * Z) + q[3]);
      o[0] += q[4] * s;
      o[1] += q[5] * s;
      o[2] += q[6] * s;
    }
    break;
  }
  default: break;
  }
  for (int d = 0; d < dim; d++) v[(size_t)p * dim + d] = o[d];
}

extern "C" int lgb_op_velocity_field(lgb_dev *d, void *stream)
{
  if (d->np <= 0 || !d->vfield) return 0;
  k_velocity_field<<<lgb_cdiv(d->np, 256), 256, 0, (cudaStream_t)stream>>>(d->np, d->g.dim, d->xp, d->alive, d->vel,
                                                                              d->vfield, d->vfield_par, d->vfield_np);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}

/* Loop scalars of InternalForwardAdvectionLoop, one thread. */
__global__ void k_ctrl(lgb_ctrl *c, int what)
{
  switch (what) {
  case LGB_CTRL_RESET_CFL:
    c->n2max_bits = 0ull;
    c->np_alive = 0;
    break;
  case LGB_CTRL_BEGIN_STEP: {
    double dt_cfl = DBL_MAX;
    if (c->n2max_bits) {
      const double n2 = __longlong_as_double((long long)(c->n2max_bits - 1ull));
      dt_cfl = c->cfl_fac * c->cfl_radius / (sqrt(n2) + 1e-16);
    }
    if (c->dt_cfl_ext > 0.0) dt_cfl = c->dt_cfl_ext;
    double dt = (c->scheme == LGB_DOPRI) ? ((c->dt_adv < dt_cfl) ? c->dt_adv : dt_cfl) : dt_cfl;
    if (c->t + dt > c->t_next) dt = c->t_next - c->t;
    c->dt = dt;
    c->dt_adv = dt; /* LagRBFSetTimeStep */
    c->maxerr_bits = 0ull;
    c->any_alive = 0;
    break;
  }
  case LGB_CTRL_DOPRI_DT: {
    /* AdvectionComputeAdaptiveTimeStep_DOPRI (dormand_prince.c:179-214) */
    double max_err = c->any_alive ? __longlong_as_double((long long)c->maxerr_bits) : -DBL_MAX;
    double fac_max = (max_err <= 1.0) ? c->dopri_fac_max : 1.0;
    double q = c->dopri_fac * pow(1.0 / max_err, 1.0 / 5.0);
    double inner = (c->dopri_fac_min < q) ? q : c->dopri_fac_min; /* PetscMax */
    double f = (fac_max < inner) ? fac_max : inner;               /* PetscMin */
    c->dopri_error = max_err;
    c->dt_adv = c->dt * f;
    break;
  }
  case LGB_CTRL_END_STEP:
    c->t += c->dt;
    c->steps += 1;
    c->particle_steps += c->np_alive;
    break;
  case LGB_CTRL_BEGIN_SWEEP:
    c->pp_left = 0;
    break;
  case LGB_CTRL_END_SWEEP: /* accepted particle steps are counted by k_pp_accept */
    if (c->pp_left == 0) c->t = c->t_next;
    c->steps += 1;
    break;
  default: break;
  }
}

__global__ void k_loop_cond(lgb_ctrl *c, cudaGraphConditionalHandle h)
{
  c->loop_iter += 1;
  const int go = c->t < c->t_next && !c->factor_error && !c->eval_error && c->loop_iter < c->loop_cap;
  cudaGraphSetConditional(h, go ? 1u : 0u);
}

extern "C" int lgb_op_loop_cond(lgb_dev *d, unsigned long long handle, void *stream)
{
  k_loop_cond<<<1, 1, 0, (cudaStream_t)stream>>>(d->ctrl, (cudaGraphConditionalHandle)handle);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}

extern "C" int lgb_op_ctrl(lgb_dev *d, int what, void *stream)
{
  k_ctrl<<<1, 1, 0, (cudaStream_t)stream>>>(d->ctrl, what);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}

/* FMA throughput probe (FP32 or FP64): 8 independent dependent-FMA chains per thread, 2 flops each. */
template <typename T>
__global__ void k_fma_probe(T *out, int iters, T a, T b)
{
  T x0 = threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)1234.5) out[0] = s; /* keep the chains alive */
}

/* Best of five event-timed launches of the probe over 4 CTAs of 512 threads per SM, in TFLOP/s. */
template <typename T>
static double fma_peak_tflops(int iters)
{
  int nsm = 0, smem = 0;
  if (lgb_device_info(&nsm, &smem)) return -1.0;
  T *out = NULL;
  if (cudaMalloc(&out, sizeof(T)) != cudaSuccess) return -1.0;
  const int threads = 512, blocks = nsm * 4;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fma_probe<T><<<blocks, threads>>>(out, 16, (T)0.999, (T)0.001); /* warm-up */
  float best = 1e30f;
  for (int r = 0; r < 5; r++) {
    cudaEventRecord(e0);
    k_fma_probe<T><<<blocks, threads>>>(out, iters, (T)0.999, (T)0.001);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    if (ms < best) best = ms;
  }
  lgb_count_launch(6);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (cudaGetLastError() != cudaSuccess) return -1.0;
  double flops = 2.0 * 8 * 16 * (double)iters * threads * blocks;
  return flops / (best * 1e-3) / 1e12;
}

extern "C" double lgb_fp32_peak_tflops(void) { return fma_peak_tflops<float>(4096); }
extern "C" double lgb_fp64_peak_tflops(void) { return fma_peak_tflops<double>(256); }
