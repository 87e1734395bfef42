/*
 * lgb_factor.cu -- batched per-patch collocation assembly, FP64 Cholesky and solve.
 *
 * Replaces the lazy patch set-up and solve of LagRBF_PartitionsSetUp (src/partitions/partition.c:
 * 384-478): PartitionAssembleRBFMatrix (partition_solve.c:47-95, partition_asmb_avx512.c:119-198),
 * MatCholeskyFactor / KSP preonly+PCCHOLESKY (partition_factor.c:37-55, partition_ksp.c:115-172) and
 * the RHS gather + MatMatSolve (partition_factor.c:57-135).
 *
 * Patches are queued by size class (LGB_NCLS classes of sizes up to 32, 64, ..., 2048 and beyond);
 * each class is one launch of a persistent grid over its work list (graph-capturable with a
 * device-side count), with the class's CTA size from the measured table (lgb_factor_tune.h), its
 * own workspace slot size (the class's largest patch) and as many CTAs as fit 1024 threads per SM
 * within the workspace budget.  The patch matrix is
 * assembled column-major into a per-CTA workspace slot (lower triangle), factored in panels of
 * CHOL_NB columns (left-looking inside a panel, then a tiled update of the trailing triangle), then
 * the F right-hand sides are solved together.  FP64 throughout: the collocation systems are
 * ill-conditioned.  A
 * non-positive pivot sets ctrl->factor_error (1-based row) and leaves the patch not set up; no
 * trap, no abort.  The factor is then "prepared" for the solves (reciprocal diagonal and scaled
 * diagonal blocks, below); when factors are kept (A_FACTOR / A_KSP) it is packed (column-major
 * lower, m(m+1)/2) so that new field values only need the two triangular solves, which run the same
 * code on the same values as the first solve.
 *
 * Roofline: FP64 pipe (m^3/3 flops per patch to factor, 2 F m^2 per solve); GB300 issues 2 DFMA
 * per clock per SM, so FP64 instructions, not bytes, are what the code counts.
 */
#include "lgb_common.cuh"

#define CHOL_NB 16 /* columns per Cholesky panel */

struct FactorParams {
  lgb_geom g;
  int F, keep;
  const int *cstart;
  const double *xs, *fs;
  const int *pm, *slot, *work;  /* work: the nodes of one patch-size class, *nwork of them */
  const int *nwork;
  const long long *coff, *foff;
  int *setup, *solved;
  double *c64, *fac, *ws;
  float *c32;
  long long ws_stride;
  lgb_ctrl *ctrl;
  double *kappa;   /* non-NULL: 1-norm condition estimate of every factored patch, by node */
};


/* Column j of the lower factor from its diagonal element down: packed column-major (m(m+1)/2,
   the kept factors) or the full column-major workspace.  L(i, j) = L[lbase(j) + (i - j)]. */
template <bool PACKED>
__device__ __forceinline__ long long lbase(int m, int j)
{
  return PACKED ? (long long)j * m - ((long long)j * (j - 1)) / 2 : (long long)j * m + j;
}
template <bool PACKED>
__device__ __forceinline__ long long lstep(int m, int j)
{
  return PACKED ? (long long)(m - j) : (long long)m + 1; /* base(j + 1) - base(j) */
}

/* The factor as the solves read it ("prepared"): the 32 x 32 diagonal blocks hold the reciprocal
   1 / L(j, j) on the diagonal and M(i, j) = L(i, j) / L(j, j) below it; every other entry is
   L(i, j).  With M the substitutions inside a diagonal block are fused multiply-adds only:
     forward   u_i = b_i - sum_{k<i} M(i,k) u_k,              y_i = u_i / L(i,i)
     backward  w_i = y_i / L(i,i) - sum_{k>i} M(k,i) x_k,      x_i = w_i
   (L(i,k) y_k = M(i,k) u_k and L(k,i) x_k / L(i,i) = M(k,i) x_k), which halves the FP64
   instructions of the block substitutions, the serial part of the solve. */
template <bool PACKED>
__device__ void prepare_diag_blocks(double *L, int m)
{
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    const long long b = lbase<PACKED>(m, j);
    const double d = L[b];
    const int iend = min((j / 32 + 1) * 32, m);
    for (int i = j + 1; i < iend; i++) L[b + (i - j)] /= d;
  }
  __syncthreads();
  for (int j = threadIdx.x; j < m; j += blockDim.x) {
    const long long b = lbase<PACKED>(m, j);
    L[b] = 1.0 / L[b];
  }
  __syncthreads();
}

/* D[r * 33 + c] = prepared diagonal block entry (j0 + r, j0 + c), r >= c; column-wise reads. */
template <bool PACKED>
__device__ __forceinline__ void stage_diag(const double *L, int m, int j0, int nb, double *D)
{
  for (int t = threadIdx.x; t < nb * nb; t += blockDim.x) {
    const int c = t / nb, r = t - c * nb;
    if (r >= c) D[r * 33 + c] = L[lbase<PACKED>(m, j0 + c) + (r - c)];
  }
}

/* Solves L L^T X = B in place for FC (1..4) columns of B (B[q*m + i]) with the prepared factor,
   in blocks of 32 rows.  Each diagonal block is staged in shared memory (D, 32 x 33) and
   substituted by one warp with shuffles, every lane issuing the same fused multiply-add (zero
   multiplier where a lane has nothing to subtract); the block's solution is kept in shared memory
   (Y, 4 x 32) and the other rows are updated by all threads, each factor element read once per
   block for all FC right-hand sides.  Forward: rows below the block, L(i, j) read down columns
   (coalesced).  Backward: rows above the block, x_i -= sum_r L(i0 + r, i) x_r, each thread
   reading 32 consecutive entries of its own column.  Only FP64 fused multiply-adds and one
   multiplication per block and right-hand side; no reductions. */
template <bool PACKED, int FC>
__device__ void chol_solve_group(const double *__restrict__ L, int m, double *B0, double *D, double *Y)
{
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nblk = (m + 31) / 32;
  for (int kb = 0; kb < nblk; kb++) {
    const int j0 = kb * 32, nb = min(32, m - j0);
    stage_diag<PACKED>(L, m, j0, nb, D);
    __syncthreads();
    if (warp == 0) {
      double u[FC];
#pragma unroll
      for (int q = 0; q < FC; q++) u[q] = (lane < nb) ? B0[(size_t)q * m + j0 + lane] : 0.0;
      for (int jj = 0; jj < nb - 1; jj++) {
        const double mij = (lane > jj && lane < nb) ? D[lane * 33 + jj] : 0.0;
#pragma unroll
        for (int q = 0; q < FC; q++) u[q] = fma(-mij, __shfl_sync(0xffffffffu, u[q], jj), u[q]);
      }
      const double rl = (lane < nb) ? D[lane * 33 + lane] : 0.0;
#pragma unroll
      for (int q = 0; q < FC; q++) {
        const double y = u[q] * rl;
        Y[q * 32 + lane] = y;
        if (lane < nb) B0[(size_t)q * m + j0 + lane] = y;
      }
    }
    __syncthreads();
    const long long b0 = lbase<PACKED>(m, j0);
    for (int i = j0 + nb + tid; i < m; i += blockDim.x) {
      double acc[FC];
#pragma unroll
      for (int q = 0; q < FC; q++) acc[q] = B0[(size_t)q * m + i];
      long long cb = b0 - j0; /* element (i, j) of column j at cb + i */
#pragma unroll 8
      for (int jj = 0; jj < nb; jj++) {
        const double l = L[cb + i - jj];
#pragma unroll
        for (int q = 0; q < FC; q++) acc[q] = fma(-l, Y[q * 32 + jj], acc[q]);
        cb += lstep<PACKED>(m, j0 + jj);
      }
#pragma unroll
      for (int q = 0; q < FC; q++) B0[(size_t)q * m + i] = acc[q];
    }
    __syncthreads();
  }
  for (int kb = nblk - 1; kb >= 0; kb--) {
    const int i0 = kb * 32, nb = min(32, m - i0);
    stage_diag<PACKED>(L, m, i0, nb, D);
    __syncthreads();
    if (warp == 0) {
      const double rl = (lane < nb) ? D[lane * 33 + lane] : 0.0;
      double w[FC];
#pragma unroll
      for (int q = 0; q < FC; q++) w[q] = ((lane < nb) ? B0[(size_t)q * m + i0 + lane] : 0.0) * rl;
      for (int ii = nb - 1; ii >= 1; ii--) {
        const double mi = (lane < ii) ? D[ii * 33 + lane] : 0.0;
#pragma unroll
        for (int q = 0; q < FC; q++) w[q] = fma(-mi, __shfl_sync(0xffffffffu, w[q], ii), w[q]);
      }
#pragma unroll
      for (int q = 0; q < FC; q++) {
        Y[q * 32 + lane] = w[q];
        if (lane < nb) B0[(size_t)q * m + i0 + lane] = w[q];
      }
    }
    __syncthreads();
    for (int i = tid; i < i0; i += blockDim.x) {
      double acc[FC];
#pragma unroll
      for (int q = 0; q < FC; q++) acc[q] = B0[(size_t)q * m + i];
      const double *ci = L + lbase<PACKED>(m, i) + (i0 - i); /* L(i0 + r, i) = ci[r] */
#pragma unroll 8
      for (int r = 0; r < nb; r++) {
        const double l = ci[r];
#pragma unroll
        for (int q = 0; q < FC; q++) acc[q] = fma(-l, Y[q * 32 + r], acc[q]);
      }
#pragma unroll
      for (int q = 0; q < FC; q++) B0[(size_t)q * m + i] = acc[q];
    }
    __syncthreads();
  }
}

/* All F right-hand sides of B (B[f*m + i]), four at a time. */
template <bool PACKED>
__device__ void chol_solve(const double *L, int m, int F, double *B, double *D, double *Y)
{
  for (int f0 = 0; f0 < F; f0 += 4) {
    double *B0 = B + (size_t)f0 * m;
    switch (min(4, F - f0)) {
    case 1: chol_solve_group<PACKED, 1>(L, m, B0, D, Y); break;
    case 2: chol_solve_group<PACKED, 2>(L, m, B0, D, Y); break;
    case 3: chol_solve_group<PACKED, 3>(L, m, B0, D, Y); break;
    default: chol_solve_group<PACKED, 4>(L, m, B0, D, Y); break;
    }
  }
}

/* ---- block reductions (blockDim.x threads; red: 32 doubles of shared memory) ---- */
__device__ double blk_reduce(double v, double *red, bool is_max)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_xor_sync(0xffffffffu, v, o);
    v = is_max ? fmax(v, u) : v + u;
  }
  __syncthreads();
  if (lane == 0) red[warp] = v;
  __syncthreads();
  double r = red[0];
  for (int w = 1; w < nw; w++) r = is_max ? fmax(r, red[w]) : r + red[w];
  return r;
}
/* Largest |z_i| and its first index. */
__device__ double blk_argmax_abs(const double *z, int m, int *idx, double *red, int *ired)
{
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  double best = -1.0;
  int bi = 0;
  for (int i = threadIdx.x; i < m; i += blockDim.x)
    if (fabs(z[i]) > best) { best = fabs(z[i]); bi = i; }
  for (int o = 16; o > 0; o >>= 1) {
    const double u = __shfl_xor_sync(0xffffffffu, best, o);
    const int ui = __shfl_xor_sync(0xffffffffu, bi, o);
    if (u > best || (u == best && ui < bi)) { best = u; bi = ui; }
  }
  __syncthreads();
  if (lane == 0) { red[warp] = best; ired[warp] = bi; }
  __syncthreads();
  best = red[0];
  bi = ired[0];
  for (int w = 1; w < nw; w++)
    if (red[w] > best || (red[w] == best && ired[w] < bi)) { best = red[w]; bi = ired[w]; }
  *idx = bi;
  return best;
}

/* ||A^-1||_1 estimate from the prepared factor in the workspace (Hager's method as refined by Higham:
   N. J. Higham, "FORTRAN codes for estimating the one-norm of a real or complex matrix", ACM TOMS 14
   (1988); A symmetric, so A^-T = A^-1): at most five iterations of x -> sign(A^-1 x) -> e_j, then
   the alternating test vector x_i = (-1)^i (1 + i/(m-1)).  v, u: two workspace vectors of m. */
__device__ double inv_norm1_estimate(const double *L, int m, double *v, double *u, double *D, double *Y, double *red,
                                     int *ired)
{
  const int tid = threadIdx.x;
  for (int i = tid; i < m; i += blockDim.x) v[i] = 1.0 / m;
  __syncthreads();
  chol_solve_group<false, 1>(L, m, v, D, Y);
  double s = 0.0;
  for (int i = tid; i < m; i += blockDim.x) s += fabs(v[i]);
  double est = blk_reduce(s, red, false);
  int jprev = -1;
  for (int it = 0; it < 5; it++) {
    for (int i = tid; i < m; i += blockDim.x) u[i] = (v[i] >= 0.0) ? 1.0 : -1.0;
    __syncthreads();
    chol_solve_group<false, 1>(L, m, u, D, Y);
    int j;
    const double zmax = blk_argmax_abs(u, m, &j, red, ired);
    double ztx;
    if (jprev < 0) {
      double t = 0.0;
      for (int i = tid; i < m; i += blockDim.x) t += u[i];
      ztx = blk_reduce(t, red, false) / m;
    } else {
      ztx = u[jprev];
    }
    if (it > 0 && zmax <= ztx) break;
    for (int i = tid; i < m; i += blockDim.x) v[i] = (i == j) ? 1.0 : 0.0;
    __syncthreads();
    chol_solve_group<false, 1>(L, m, v, D, Y);
    s = 0.0;
    for (int i = tid; i < m; i += blockDim.x) s += fabs(v[i]);
    const double e2 = blk_reduce(s, red, false);
    if (e2 <= est) break;
    est = e2;
    jprev = j;
  }
  for (int i = tid; i < m; i += blockDim.x) v[i] = ((i & 1) ? -1.0 : 1.0) * (1.0 + (m > 1 ? (double)i / (m - 1) : 0.0));
  __syncthreads();
  chol_solve_group<false, 1>(L, m, v, D, Y);
  s = 0.0;
  for (int i = tid; i < m; i += blockDim.x) s += fabs(v[i]);
  const double alt = 2.0 * blk_reduce(s, red, false) / (3.0 * m);
  return fmax(est, alt);
}

/* One template per CTA size NT (the patch-size class's entry of the tuning table). */
template <int NT>
__global__ void __launch_bounds__(NT) k_factor(FactorParams P)
{
  __shared__ int s_cstart[8], s_cnt[8], s_off[8];
  __shared__ int s_fail;
  __shared__ double s_rd;
  __shared__ double s_diag[32 * 33], s_y[4 * 32];
  __shared__ double s_red[32];
  __shared__ int s_ired[32];
  const lgb_geom &g = P.g;
  const int nwork = *P.nwork;
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
    for (int q = tid; q < m; q += NT) {
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
        for (int i = j + tid; i < m; i += NT) {
          double dx = X[(size_t)i * g.dim] - xj0, dy = X[(size_t)i * g.dim + 1] - xj1, d2;
          if (g.dim == 3) {
            double dz = X[(size_t)i * g.dim + 2] - xj2;
            d2 = fma(dx, dx, fma(dy, dy, dz * dz));
          } else d2 = fma(dx, dx, dy * dy);
          A[(size_t)j * m + i] = lgb_phi<double>(g.kernel, sqrt(d2), eps);
        }
      }
      __syncthreads();
      /* 1-norm of the symmetric matrix (largest column sum of |A|) for the condition estimate */
      double anorm = 0.0;
      if (P.kappa) {
        double cm = 0.0;
        for (int j = tid; j < m; j += NT) {
          double cs = 0.0;
          for (int i = j; i < m; i++) cs += fabs(A[(size_t)j * m + i]);
          for (int k = 0; k < j; k++) cs += fabs(A[(size_t)k * m + j]);
          cm = fmax(cm, cs);
        }
        anorm = blk_reduce(cm, s_red, true);
      }
      /* Cholesky in panels of CHOL_NB columns: each panel is factored left-looking from the
         entries already updated by the earlier panels, then the trailing lower triangle is updated
         by the panel (tiles of 32 x 32, one warp per tile).  Every entry receives its updates
         -L(i,k) L(j,k) one at a time in ascending k, exactly as in an unblocked left-looking
         factorisation, so the factor is the same bit for bit; the blocking only stops each column
         from re-reading all earlier columns. */
      double *Ps = B + (size_t)m * F; /* panel rows [p0, m) x CHOL_NB, stride CHOL_NB + 1 */
      for (int p0 = 0; p0 < m && !s_fail; p0 += CHOL_NB) {
        const int nb = min(CHOL_NB, m - p0), p1 = p0 + nb;
        for (int j = p0; j < p1; j++) {
          const double *Lj = A + j; /* row j: Lj[k*m] = L(j,k) */
          for (int i = j + tid; i < m; i += NT) {
            double s = A[(size_t)j * m + i];
            for (int k = p0; k < j; k++) s -= A[(size_t)k * m + i] * Lj[(size_t)k * m];
            A[(size_t)j * m + i] = s;
          }
          __syncthreads();
          /* one thread takes the pivot's square root and its reciprocal; the column is scaled by
             multiplication (an FP64 division per entry would cost the FP64 pipe ~10 operations) */
          if (tid == 0) {
            const double dd = A[(size_t)j * m + j];
            if (!(dd > 0.0)) {
              if (atomicCAS(&P.ctrl->factor_error, 0, j + 1) == 0) P.ctrl->factor_node = node;
              s_fail = 1;
            } else {
              const double sd = sqrt(dd);
              A[(size_t)j * m + j] = sd;
              s_rd = 1.0 / sd;
            }
          }
          __syncthreads();
          if (s_fail) break;
          const double rd = s_rd;
          for (int i = j + 1 + tid; i < m; i += NT) A[(size_t)j * m + i] *= rd;
          __syncthreads();
        }
        __syncthreads();
        if (s_fail || p1 >= m) break;
        /* stage the panel's rows (row-major, padded) for the trailing update */
        for (int t = tid; t < (m - p0) * nb; t += NT) {
          const int kk = t / (m - p0), r = t - kk * (m - p0);
          Ps[(size_t)r * (CHOL_NB + 1) + kk] = A[(size_t)(p0 + kk) * m + p0 + r];
        }
        __syncthreads();
        const int T = (m - p1 + 31) / 32, ntile = T * (T + 1) / 2;
        const int lane = tid & 31, warp = tid >> 5;
        for (int t = warp; t < ntile; t += NT / 32) {
          int c = 0, rem = t;
          while (rem >= T - c) { rem -= T - c; c++; }
          const int i = p1 + 32 * (c + rem) + lane, jb = p1 + 32 * c;
          if (i >= m) continue;
          double li[CHOL_NB];
#pragma unroll
          for (int kk = 0; kk < CHOL_NB; kk++) li[kk] = (kk < nb) ? Ps[(size_t)(i - p0) * (CHOL_NB + 1) + kk] : 0.0;
          const int jend = min(jb + 32, i + 1);
          for (int j = jb; j < jend; j++) {
            const double *lj = Ps + (size_t)(j - p0) * (CHOL_NB + 1);
            double a = A[(size_t)j * m + i];
#pragma unroll
            for (int kk = 0; kk < CHOL_NB; kk++)
              if (kk < nb) a -= li[kk] * lj[kk];
            A[(size_t)j * m + i] = a;
          }
        }
        __syncthreads();
      }
      __syncthreads();
      if (s_fail) { __syncthreads(); continue; }
      prepare_diag_blocks<false>(A, m);
      if (P.kappa) {
        const double inv = inv_norm1_estimate(A, m, Ps, Ps + m, s_diag, s_y, s_red, s_ired);
        if (tid == 0) P.kappa[node] = anorm * inv;
      }
      if (P.keep) {
        double *Fk = P.fac + P.foff[node];
        for (int j = 0; j < m; j++) {
          long long base = (long long)j * m - ((long long)j * (j - 1)) / 2; /* packed column j */
          for (int i = j + tid; i < m; i += NT) Fk[base + (i - j)] = A[(size_t)j * m + i];
        }
      }
      if (tid == 0) {
        atomicAdd(&P.ctrl->factor_flops, (double)m * m * m / 3.0 + 2.0 * (double)m * m * F);
        atomicAdd(&P.ctrl->nfactored, 1);
      }
    } else if (m > 0) {
      if (tid == 0) atomicAdd(&P.ctrl->factor_flops, 2.0 * (double)m * m * F);
    }
    __syncthreads();
    if (m > 0) {
      if (have_factor) chol_solve<true>(P.fac + P.foff[node], m, F, B, s_diag, s_y);
      else chol_solve<false>(A, m, F, B, s_diag, s_y);
      /* coefficients [point][field] in both precisions */
      const long long c0 = P.coff[node];
      for (int q = tid; q < m; q += NT)
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
  if (d->nws <= 0 || !d->ws) return 0;
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
  P.kappa = d->cond_on ? d->kappa : NULL;
  /* one launch per patch-size class holding patches: its CTA size, grid and workspace slots */
  for (int c = 0; c < LGB_NCLS; c++) {
    if (d->cls_cap[c] <= 0 || d->cls_grid[c] <= 0) continue;
    P.work = d->work + d->cls_off[c];
    P.nwork = &d->ctrl->nwork_c[c];
    P.ws_stride = d->cls_stride[c];
    cudaStream_t s = (cudaStream_t)stream;
    switch (d->cls_threads[c]) {
    case 32: k_factor<32><<<d->cls_grid[c], 32, 0, s>>>(P); break;
    case 64: k_factor<64><<<d->cls_grid[c], 64, 0, s>>>(P); break;
    case 256: k_factor<256><<<d->cls_grid[c], 256, 0, s>>>(P); break;
    default: k_factor<128><<<d->cls_grid[c], 128, 0, s>>>(P); break;
    }
    lgb_count_launch(1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
  }
  return 0;
}
