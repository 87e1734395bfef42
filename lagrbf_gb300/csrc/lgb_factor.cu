/*
 * lgb_factor.cu -- batched per-patch collocation assembly, FP64 Cholesky and solve.
 *
 * Replaces the lazy patch set-up and solve of LagRBF_PartitionsSetUp (src/partitions/partition.c:
 * 384-478): PartitionAssembleRBFMatrix (partition_solve.c:47-95, partition_asmb_avx512.c:119-198),
 * MatCholeskyFactor / KSP preonly+PCCHOLESKY (partition_factor.c:37-55, partition_ksp.c:115-172) and
 * the RHS gather + MatMatSolve (partition_factor.c:57-135).
 *
 * One CTA per queued patch (persistent grid over the work list, so the launch is graph-capturable
 * with a device-side count).  The patch matrix is assembled column-major into a per-CTA workspace
 * slot (lower triangle), factored left-looking one column at a time (every thread owns rows, the
 * reads of a column are coalesced and the pivot row is a broadcast), then the F right-hand sides
 * are solved together.  FP64 throughout: the collocation systems are ill-conditioned.  A
 * non-positive pivot sets ctrl->factor_error (1-based row) and leaves the patch not set up; no
 * trap, no abort.  When factors are kept (A_FACTOR / A_KSP) the factor is packed (column-major
 * lower, m(m+1)/2) so that new field values only need the two triangular solves.
 *
 * Roofline: FP64 pipe (m^3/3 flops per patch); workspace traffic stays in L2 for m <= ~700.
 */
#include "lgb_common.cuh"

#define FACT_T 256

struct FactorParams {
  lgb_geom g;
  int F, keep;
  const int *cstart;
  const double *xs, *fs;
  const int *pm, *slot, *work;
  const long long *coff, *foff;
  int *setup, *solved;
  double *c64, *fac, *ws;
  float *c32;
  long long ws_stride;
  lgb_ctrl *ctrl;
};

__device__ __forceinline__ double block_sum(double v, double *red)
{
  for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
  int w = threadIdx.x >> 5, l = threadIdx.x & 31;
  __syncthreads();
  if (l == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (threadIdx.x < 32) {
    s = (threadIdx.x < FACT_T / 32) ? red[threadIdx.x] : 0.0;
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
  }
  if (threadIdx.x == 0) red[FACT_T / 32] = s;
  __syncthreads();
  return red[FACT_T / 32];
}

__global__ void __launch_bounds__(FACT_T) k_factor(FactorParams P)
{
  __shared__ int s_cstart[8], s_cnt[8], s_off[8];
  __shared__ double red[FACT_T / 32 + 1];
  __shared__ int s_fail;
  const lgb_geom &g = P.g;
  const int nwork = P.ctrl->nwork;
  const int tid = threadIdx.x;
  double *A = P.ws + (size_t)blockIdx.x * P.ws_stride;
  for (int w = blockIdx.x; w < nwork; w += gridDim.x) {
    const int node = P.work[w];
    const int m = P.pm[node];
    const int F = P.F;
    if (tid == 0) {
      int nxy = g.n[0] * g.n[1];
      int l = node / nxy, r = node - l * nxy, j = r / g.n[0], i = r - j * g.n[0];
      for (int s = 0; s < 8; s++) {
        int dx = s & 1, dy = (s >> 1) & 1, dz = (s >> 2) & 1;
        int ci = i - 1 + dx, cj = j - 1 + dy, cl = (g.dim == 3) ? (l - 1 + dz) : 0;
        bool ok = (g.dim == 3 || dz == 0) && ci >= 0 && ci < g.nc[0] && cj >= 0 && cj < g.nc[1] && cl >= 0 &&
                  cl < g.nc[2];
        int c = ok ? ci + cj * g.nc[0] + cl * g.nc[0] * g.nc[1] : 0;
        s_cstart[s] = ok ? P.cstart[c] : 0;
        s_cnt[s] = ok ? P.cstart[c + 1] - P.cstart[c] : 0;
        s_off[s] = P.slot[node * 8 + s];
      }
      s_fail = 0;
    }
    __syncthreads();
    double *X = A + (size_t)m * m;     /* m*dim patch coordinates */
    double *B = X + (size_t)m * g.dim; /* m*F right-hand sides / solutions */
    /* gather the patch points (reference patch order) and their values */
    for (int q = tid; q < m; q += FACT_T) {
      int s = 0;
      while (s < 7 && q >= s_off[s] + s_cnt[s]) s++;
      int src = s_cstart[s] + (q - s_off[s]);
      for (int d = 0; d < g.dim; d++) X[(size_t)q * g.dim + d] = P.xs[(size_t)src * g.dim + d];
      for (int f = 0; f < F; f++) B[(size_t)f * m + q] = P.fs[(size_t)src * F + f];
    }
    __syncthreads();
    const bool have_factor = P.setup[node] && P.keep;
    if (m > 0 && !have_factor) {
      /* assemble the lower triangle, column-major: A[j*m + i], i >= j */
      const double eps = g.eps_r;
      for (int j = 0; j < m; j++) {
        const double xj0 = X[(size_t)j * g.dim], xj1 = X[(size_t)j * g.dim + 1];
        const double xj2 = (g.dim == 3) ? X[(size_t)j * g.dim + 2] : 0.0;
        for (int i = j + tid; i < m; i += FACT_T) {
          double dx = X[(size_t)i * g.dim] - xj0, dy = X[(size_t)i * g.dim + 1] - xj1, d2;
          if (g.dim == 3) {
            double dz = X[(size_t)i * g.dim + 2] - xj2;
            d2 = fma(dx, dx, fma(dy, dy, dz * dz));
          } else d2 = fma(dx, dx, dy * dy);
          A[(size_t)j * m + i] = lgb_phi<double>(g.kernel, sqrt(d2), eps);
        }
      }
      __syncthreads();
      /* left-looking Cholesky */
      for (int j = 0; j < m; j++) {
        const double *Lj = A + j; /* row j: Lj[k*m] = L(j,k) */
        for (int i = j + tid; i < m; i += FACT_T) {
          double s = A[(size_t)j * m + i];
          for (int k = 0; k < j; k++) s -= A[(size_t)k * m + i] * Lj[(size_t)k * m];
          A[(size_t)j * m + i] = s;
        }
        __syncthreads();
        double dd = A[(size_t)j * m + j];
        if (!(dd > 0.0)) {
          if (tid == 0) {
            if (atomicCAS(&P.ctrl->factor_error, 0, j + 1) == 0) P.ctrl->factor_node = node;
            s_fail = 1;
          }
          break;
        }
        dd = sqrt(dd);
        for (int i = j + 1 + tid; i < m; i += FACT_T) A[(size_t)j * m + i] /= dd;
        __syncthreads();
        if (tid == 0) A[(size_t)j * m + j] = dd;
        __syncthreads();
      }
      __syncthreads();
      if (s_fail) { __syncthreads(); continue; }
      if (P.keep) {
        double *Fk = P.fac + P.foff[node];
        for (int j = 0; j < m; j++) {
          long long base = (long long)j * m - ((long long)j * (j - 1)) / 2; /* packed column j */
          for (int i = j + tid; i < m; i += FACT_T) Fk[base + (i - j)] = A[(size_t)j * m + i];
        }
      }
      if (tid == 0) {
        atomicAdd(&P.ctrl->factor_flops, (double)m * m * m / 3.0 + 2.0 * (double)m * m * F);
        atomicAdd(&P.ctrl->nfactored, 1);
      }
    } else if (m > 0) {
      const double *Fk = P.fac + P.foff[node];
      for (int j = 0; j < m; j++) {
        long long base = (long long)j * m - ((long long)j * (j - 1)) / 2;
        for (int i = j + tid; i < m; i += FACT_T) A[(size_t)j * m + i] = Fk[base + (i - j)];
      }
      if (tid == 0) atomicAdd(&P.ctrl->factor_flops, 2.0 * (double)m * m * F);
    }
    __syncthreads();
    if (m > 0) {
      /* forward: L y = b (column sweep, coalesced column reads) */
      for (int j = 0; j < m; j++) {
        const double ljj = A[(size_t)j * m + j];
        for (int f = 0; f < F; f++) {
          double yj = B[(size_t)f * m + j] / ljj;
          for (int i = j + 1 + tid; i < m; i += FACT_T) B[(size_t)f * m + i] -= A[(size_t)j * m + i] * yj;
        }
        __syncthreads();
        if (tid == 0)
          for (int f = 0; f < F; f++) B[(size_t)f * m + j] /= ljj;
        __syncthreads();
      }
      /* backward: L^T x = y (dot products with column i) */
      for (int i = m - 1; i >= 0; i--) {
        const double lii = A[(size_t)i * m + i];
        for (int f = 0; f < F; f++) {
          double part = 0.0;
          for (int k = i + 1 + tid; k < m; k += FACT_T) part += A[(size_t)i * m + k] * B[(size_t)f * m + k];
          double sum = block_sum(part, red);
          if (tid == 0) B[(size_t)f * m + i] = (B[(size_t)f * m + i] - sum) / lii;
          __syncthreads();
        }
      }
      /* coefficients [point][field] in both precisions */
      const long long c0 = P.coff[node];
      for (int q = tid; q < m; q += FACT_T)
        for (int f = 0; f < F; f++) {
          double v = B[(size_t)f * m + q];
          P.c64[(size_t)(c0 + q) * F + f] = v;
          P.c32[(size_t)(c0 + q) * F + f] = (float)v;
        }
    }
    __syncthreads();
    if (tid == 0) {
      P.setup[node] = 1;
      P.solved[node] = 1;
    }
    __syncthreads();
  }
}

extern "C" int lgb_op_factor(lgb_dev *d, void *stream)
{
  if (d->nws <= 0) return 0;
  FactorParams P;
  P.g = d->g;
  P.F = d->F;
  P.keep = d->keep_factors;
  P.cstart = d->cstart;
  P.xs = d->xs;
  P.fs = d->fs;
  P.pm = d->pm;
  P.slot = d->slot;
  P.work = d->work;
  P.coff = d->coff;
  P.foff = d->foff;
  P.setup = d->setup;
  P.solved = d->solved;
  P.c64 = d->c64;
  P.c32 = d->c32;
  P.fac = d->fac;
  P.ws = d->ws;
  P.ws_stride = d->ws_stride;
  P.ctrl = d->ctrl;
  k_factor<<<d->nws, FACT_T, 0, (cudaStream_t)stream>>>(P);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}
