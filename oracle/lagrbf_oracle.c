/*
 * lagrbf_oracle.c -- CPU restatement of LagRBF's PU-RBF interpolation and advection path.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker, CPU baseline).  See lagrbf_oracle.h for the
 * parity status and the conventions fixed where the reference delegates to PETSc.
 *
 * Build without fast-math and with -ffp-contract=off so that every fma() below is the only
 * fused operation: the association of sums follows the reference's vector code (8-lane chunks
 * in interpolation_avx512.c, 4-lane chunks in weights_avx.c) and stays identical on x86-64 and
 * aarch64.
 */
#include "lagrbf_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <float.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_MAX_REAL DBL_MAX
#define ORC_MIN(a, b) (((a) < (b)) ? (a) : (b)) /* PetscMin */
#define ORC_MAX(a, b) (((a) < (b)) ? (b) : (a)) /* PetscMax */

/* Error codes follow PETSc's numbering for the analogous failures. */
#define ORC_ERR_ARG_SIZ 60
#define ORC_ERR_ARG_WRONG 62
#define ORC_ERR_ARG_OUTOFRANGE 63
#define ORC_ERR_ARG_WRONGSTATE 73
#define ORC_ERR_PLIB 77
#define ORC_ERR_MAT_CH_ZRPVT 81
#define ORC_ERR_ARG_NULL 85
#define ORC_ERR_MEM 55
#define ORC_ERR_SUP 56

/* ======================================================================================= */
/* configuration                                                                            */
/* ======================================================================================= */
void orc_config_default(orc_config *cfg)
{
  memset(cfg, 0, sizeof(*cfg));
  cfg->dim = 3;
  cfg->n[0] = cfg->n[1] = cfg->n[2] = 4;
  cfg->O[0] = cfg->O[1] = cfg->O[2] = 0.0;
  cfg->L[0] = cfg->L[1] = cfg->L[2] = 1.0;
  cfg->overlap = 1.0;                 /* partition_of_unity.c:103 */
  cfg->shape_factor = 1.0;            /* partition_of_unity.c:58 */
  cfg->kernel = ORC_KERNEL_LINEAR;    /* lagrangian_rbf.c:47 */
  cfg->solve_method = ORC_A_FACTOR;   /* lagrangian_rbf.c:63 */
  cfg->nfields = 0;
  cfg->advection = 0;
  cfg->scheme = ORC_DOPRI;            /* lagrangian_rbf.c:186 */
  cfg->cfl_fac = 0.4;                 /* lagrangian_rbf.c:58 */
  cfg->dt = 1e-10;                    /* advection_ctx.c:62 */
  cfg->rmin = 0.0;
  cfg->rmax = ORC_MAX_REAL;
  cfg->dopri_dt_fac = 0.9;            /* dormand_prince.c:318-322 */
  cfg->dopri_dt_fac_min = 1.0e-2;
  cfg->dopri_dt_fac_max = 1.0e2;
  cfg->dopri_atol = 1.0e-3;
  cfg->dopri_rtol = 1.0e-3;
}

/* ======================================================================================= */
/* geometry                                                                                 */
/* ======================================================================================= */
void orc_pu_setup(orc_pu *pu, const orc_config *cfg)
{
  int d;
  double box_length = 0.0, overlap, radius;
  memset(pu, 0, sizeof(*pu));
  pu->dim = cfg->dim;
  pu->nnodes = 1;
  pu->ncells = 1;
  for (d = 0; d < 3; d++) {
    if (d < cfg->dim) {
      pu->n[d] = cfg->n[d];
      pu->O[d] = cfg->O[d];
      pu->L[d] = cfg->L[d];
      pu->h[d] = (pu->L[d] - pu->O[d]) / (double)(pu->n[d] - 1); /* DMDASetUniformCoordinates */
    } else {
      pu->n[d] = 1; pu->O[d] = 0.0; pu->L[d] = 0.0; pu->h[d] = 1.0;
    }
  }
  for (d = 0; d < cfg->dim; d++) { pu->nnodes *= pu->n[d]; pu->ncells *= (pu->n[d] - 1); }
  pu->nen = 1 << cfg->dim;
  /* PartitionOfUnityComputeSupport, partition_of_unity.c:322-346 */
  for (d = 0; d < cfg->dim; d++) box_length = ORC_MAX(box_length, (pu->L[d] - pu->O[d]));
  overlap = cfg->overlap * box_length;
  radius = overlap / pow((double)pu->nnodes, 1.0 / cfg->dim);
  pu->eps_w = 1.0 / radius;
  /* PartitionOfUnityComputeShapeFactor, partition_of_unity.c:348-355 */
  pu->eps_r = cfg->shape_factor * pu->eps_w;
}

static inline double node_coord(const orc_pu *pu, int d, int i) { return pu->O[d] + pu->h[d] * i; }

int orc_cell_corner(const orc_pu *pu, int cell, int k)
{
  /* PETSc Q1 element node order: counter-clockwise on the lower face, then the upper face. */
  static const int off2[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
  static const int off3[8][3] = {{0, 0, 0}, {1, 0, 0}, {1, 1, 0}, {0, 1, 0},
                                 {0, 0, 1}, {1, 0, 1}, {1, 1, 1}, {0, 1, 1}};
  int cx = pu->n[0] - 1, cy = pu->n[1] - 1;
  int i, j, l;
  if (pu->dim == 2) {
    j = cell / cx; i = cell - j * cx;
    return (i + off2[k][0]) + (j + off2[k][1]) * pu->n[0];
  }
  l = cell / (cx * cy); j = (cell - l * cx * cy) / cx; i = cell - l * cx * cy - j * cx;
  return (i + off3[k][0]) + (j + off3[k][1]) * pu->n[0] + (l + off3[k][2]) * pu->n[0] * pu->n[1];
}

/* ======================================================================================= */
/* RBF kernels, kernels_rbf.c:31-91 (scalar) and kernels_rbf_avx512.h / _avx.h (lane form)  */
/* ======================================================================================= */
double orc_phi_scalar(int kernel, double r, double eps)
{
  double u;
  switch (kernel) {
  case ORC_KERNEL_LINEAR: return eps * r;
  case ORC_KERNEL_WENDLAND_C0: u = 1.0 - eps * r; if (u < 0.0) return 0.0; return u * u;
  case ORC_KERNEL_WENDLAND_C2: u = 1.0 - eps * r; if (u < 0.0) return 0.0; return pow(u, 4) * (5.0 - 4.0 * u);
  case ORC_KERNEL_BUMP: u = 1.0 - eps * r; if (u < 0.0) return 0.0; return exp(-1.0 / (u * (2.0 - u)));
  case ORC_KERNEL_MQ: u = eps * r; return sqrt(1.0 + u * u);
  case ORC_KERNEL_IMQ: u = eps * r; return 1.0 / sqrt(1.0 + u * u);
  case ORC_KERNEL_GAUSSIAN: u = eps * r; return exp(-u * u);
  default: return NAN;
  }
}

/* One lane of the vector kernels (same operation order as the intrinsics).  The reference's
   vector exp (exp_avx.h) is a polynomial approximation; libm exp stands in for it, so the
   Gaussian and bump kernels agree with the reference to about one ulp, not bit for bit. */
static inline double phi_lane(int kernel, double r, double eps)
{
  double u, u2, u4, inner;
  switch (kernel) {
  case ORC_KERNEL_LINEAR: return eps * r;
  case ORC_KERNEL_WENDLAND_C0: u = 1.0 - eps * r; if (!(u >= 0.0)) u = 0.0; return u * u;
  case ORC_KERNEL_WENDLAND_C2:
    /* the mask select of the vector form, without a branch (so loops over lanes stay loops) */
    u = 1.0 - eps * r;
    u2 = u * u; u4 = u2 * u2; inner = 5.0 - 4.0 * u;
    return (u >= 0.0) ? u4 * inner : 0.0;
  case ORC_KERNEL_BUMP:
    u = 1.0 - eps * r;
    if (!(u >= 0.0)) return 0.0;
    return exp(-1.0 / (u * (2.0 - u)));
  case ORC_KERNEL_GAUSSIAN: u = eps * r; u2 = u * u; return exp(u2 * -1.0);
  default: return orc_phi_scalar(kernel, r, eps); /* MQ / IMQ have no vector form */
  }
}

double orc_phi_lane(int kernel, double r, double eps) { return phi_lane(kernel, r, eps); }

/* ======================================================================================= */
/* binning                                                                                  */
/* ======================================================================================= */
/* Convention (PETSc DMLocatePoints on the uniform DMDA is not vendored): cell index per axis is
   floor((x - O)/h), with x == L assigned to the last cell; a coordinate outside [O, L] (or NaN)
   is not located (-1). */
static inline int locate_one(const orc_pu *pu, const double *x)
{
  int d, c[3] = {0, 0, 0};
  for (d = 0; d < pu->dim; d++) {
    double t;
    if (!(x[d] >= pu->O[d] && x[d] <= pu->L[d])) return -1;
    t = floor((x[d] - pu->O[d]) / pu->h[d]);
    c[d] = (int)t;
    if (c[d] > pu->n[d] - 2) c[d] = pu->n[d] - 2;
    if (c[d] < 0) c[d] = 0;
  }
  if (pu->dim == 2) return c[0] + c[1] * (pu->n[0] - 1);
  return c[0] + c[1] * (pu->n[0] - 1) + c[2] * (pu->n[0] - 1) * (pu->n[1] - 1);
}

void orc_locate(const orc_pu *pu, int np, const double *coords, int *cellid)
{
  int p;
  for (p = 0; p < np; p++) cellid[p] = locate_one(pu, &coords[pu->dim * p]);
}

void orc_cell_csr(const orc_pu *pu, int np, const int *cellid, int *cell_start, int *cell_pts)
{
  int c, p;
  int *fill = (int *)calloc((size_t)pu->ncells + 1, sizeof(int));
  for (c = 0; c <= pu->ncells; c++) cell_start[c] = 0;
  for (p = 0; p < np; p++) if (cellid[p] >= 0) cell_start[cellid[p] + 1]++;
  for (c = 0; c < pu->ncells; c++) cell_start[c + 1] += cell_start[c];
  for (p = 0; p < np; p++) {
    int cc = cellid[p];
    if (cc < 0) continue;
    cell_pts[cell_start[cc] + fill[cc]++] = p;
  }
  free(fill);
}

/* Inverse map node -> adjacent cells, in ascending cell order (partition.c:54-87). */
static void node_cells(const orc_pu *pu, int *nc_start, int *nc_list)
{
  int e, k, n;
  int *fill = (int *)calloc((size_t)pu->nnodes, sizeof(int));
  for (n = 0; n <= pu->nnodes; n++) nc_start[n] = 0;
  for (e = 0; e < pu->ncells; e++)
    for (k = 0; k < pu->nen; k++) nc_start[orc_cell_corner(pu, e, k) + 1]++;
  for (n = 0; n < pu->nnodes; n++) nc_start[n + 1] += nc_start[n];
  for (e = 0; e < pu->ncells; e++)
    for (k = 0; k < pu->nen; k++) {
      int nd = orc_cell_corner(pu, e, k);
      nc_list[nc_start[nd] + fill[nd]++] = e;
    }
  free(fill);
}

long orc_patch_csr(const orc_pu *pu, const int *cell_start, const int *cell_pts, int *patch_start, int *patch_pts)
{
  int n, q;
  long off = 0;
  int *nc_start = (int *)malloc(sizeof(int) * ((size_t)pu->nnodes + 1));
  int *nc_list = (int *)malloc(sizeof(int) * ((size_t)pu->ncells * pu->nen));
  node_cells(pu, nc_start, nc_list);
  for (n = 0; n < pu->nnodes; n++) {
    if (patch_start) patch_start[n] = (int)off;
    for (q = nc_start[n]; q < nc_start[n + 1]; q++) {
      int c = nc_list[q];
      int cnt = cell_start[c + 1] - cell_start[c];
      if (patch_pts) memcpy(&patch_pts[off], &cell_pts[cell_start[c]], sizeof(int) * (size_t)cnt);
      off += cnt;
    }
  }
  if (patch_start) patch_start[pu->nnodes] = (int)off;
  free(nc_start); free(nc_list);
  return off;
}

long orc_block_csr(const orc_pu *pu, const int *cell_start, const int *cell_pts, int *blk_start, int *blk_pts)
{
  int cx = pu->n[0] - 1, cy = pu->n[1] - 1, cz = (pu->dim == 3) ? pu->n[2] - 1 : 1;
  int c;
  long off = 0;
  for (c = 0; c < pu->ncells; c++) {
    int l = c / (cx * cy), j = (c - l * cx * cy) / cx, i = c - l * cx * cy - j * cx;
    int dz, dy, dx, zlo = (pu->dim == 3) ? -1 : 0, zhi = (pu->dim == 3) ? 1 : 0;
    if (blk_start) blk_start[c] = (int)off;
    /* neighbour order of CellInfoCreateNeighbourElements_{2D,3D}: ascending linear offset */
    for (dz = zlo; dz <= zhi; dz++)
      for (dy = -1; dy <= 1; dy++)
        for (dx = -1; dx <= 1; dx++) {
          int ii = i + dx, jj = j + dy, ll = l + dz, nb, cnt;
          if (ii < 0 || ii >= cx || jj < 0 || jj >= cy || ll < 0 || ll >= cz) continue;
          nb = ii + jj * cx + ll * cx * cy;
          cnt = cell_start[nb + 1] - cell_start[nb];
          if (blk_pts) memcpy(&blk_pts[off], &cell_pts[cell_start[nb]], sizeof(int) * (size_t)cnt);
          off += cnt;
        }
  }
  if (blk_start) blk_start[pu->ncells] = (int)off;
  return off;
}

/* ======================================================================================= */
/* PU weights: SwarmInterpSetWeights_AVX256 (weights_avx.c:97-243)                          */
/* ======================================================================================= */
/* Node coordinates as the DMDA coordinate vector holds them (LA_coords, weights_avx.c:122-125):
   node n = ix + iy*nx + iz*nx*ny at O + h*i per axis (partition_of_unity.c:143). */
static double *node_table(const orc_pu *pu)
{
  int n, d;
  double *t = (double *)malloc(sizeof(double) * (size_t)pu->dim * (size_t)pu->nnodes);
  if (!t) return NULL;
  for (n = 0; n < pu->nnodes; n++) {
    int idx[3];
    idx[0] = n % pu->n[0];
    idx[1] = (n / pu->n[0]) % pu->n[1];
    idx[2] = n / (pu->n[0] * pu->n[1]);
    for (d = 0; d < pu->dim; d++) t[(size_t)pu->dim * n + d] = node_coord(pu, d, idx[d]);
  }
  return t;
}

static inline double wdist_lane(int dim, const double *x, const double *c)
{
  double dx = x[0] - c[0], dy = x[1] - c[1];
  if (dim == 2) return sqrt(fma(dx, dx, dy * dy));
  {
    double dz = x[2] - c[2];
    return sqrt(fma(dx, dx, fma(dy, dy, dz * dz)));
  }
}

static inline double wdist_scalar(int dim, const double *x, const double *c)
{
  int d;
  double dist = 0.0;
  for (d = 0; d < dim; d++) dist += (x[d] - c[d]) * (x[d] - c[d]);
  return sqrt(dist);
}

static inline __attribute__((always_inline)) void weights_one_d(const orc_pu *pu, const int dim,
                                                                 const double *ntab, const double *x, int cell,
                                                                 double *w)
{
  int nen = pu->nen, k, n, l;
  int corners[8];
  int aligned = (pu->nnodes / 4) * 4;
  double sum_w = 0.0;
  for (k = 0; k < nen; k++) corners[k] = orc_cell_corner(pu, cell, k);
  for (n = 0; n < aligned; n += 4) {
    double wa[4];
    for (l = 0; l < 4; l++)
      wa[l] = phi_lane(ORC_KERNEL_WENDLAND_C2, wdist_lane(dim, x, &ntab[(size_t)dim * (n + l)]), pu->eps_w);
    sum_w += wa[0] + wa[1] + wa[2] + wa[3];
    for (k = 0; k < nen; k++) {
      int nd = corners[k];
      if (nd == n) w[k] = wa[0];
      else if (nd == n + 1) w[k] = wa[1];
      else if (nd == n + 2) w[k] = wa[2];
      else if (nd == n + 3) w[k] = wa[3];
    }
  }
  for (; n < pu->nnodes; n++) {
    double weight = orc_phi_scalar(ORC_KERNEL_WENDLAND_C2, wdist_scalar(dim, x, &ntab[(size_t)dim * n]), pu->eps_w);
    sum_w += weight;
    for (k = 0; k < nen; k++) if (corners[k] == n) { w[k] = weight; break; }
  }
  for (k = 0; k < nen; k++) {
    if (sum_w > 0.0) w[k] /= sum_w;
    else w[k] = 0.0;
  }
}

static void weights_one(const orc_pu *pu, const double *ntab, const double *x, int cell, double *w)
{
  if (pu->dim == 2) weights_one_d(pu, 2, ntab, x, cell, w);
  else weights_one_d(pu, 3, ntab, x, cell, w);
}

void orc_weights(const orc_pu *pu, int np, const double *coords, const int *cellid, const int *alive,
                 double *weights)
{
  int p;
  double *ntab = node_table(pu);
  if (!ntab) return;
  for (p = 0; p < np; p++) {
    if (alive && !alive[p]) continue;
    if (cellid[p] < 0) continue;
    weights_one(pu, ntab, &coords[pu->dim * p], cellid[p], &weights[pu->nen * p]);
  }
  free(ntab);
}

/* ======================================================================================= */
/* patch assembly, factorisation and solve                                                  */
/* ======================================================================================= */
static inline double adist_lane(int dim, const double *xi, const double *xj)
{
  double dx = xi[0] - xj[0], dy = xi[1] - xj[1];
  if (dim == 2) return sqrt(fma(dx, dx, dy * dy));
  {
    double dz = xi[2] - xj[2];
    return sqrt(fma(dx, dx, fma(dy, dy, dz * dz)));
  }
}

static inline double adist_scalar(int dim, const double *xi, const double *xj)
{
  int d;
  double dist = 0.0;
  for (d = 0; d < dim; d++) dist += (xi[d] - xj[d]) * (xi[d] - xj[d]);
  return sqrt(dist);
}

/* PartitionAssembleRBFMatrix_AVX512, partition_asmb_avx512.c:119-198 (row-major, symmetric). */
static void assemble(const orc_pu *pu, int kernel, int m, const int *idx, const double *coords, double *A)
{
  int i, j, k, dim = pu->dim;
  double eps = pu->eps_r;
  for (i = 0; i < m; i++) {
    const double *xi = &coords[dim * idx[i]];
    for (j = i; j < (m - 7); j += 8) {
      for (k = 0; k < 8; k++) {
        double v = phi_lane(kernel, adist_lane(dim, xi, &coords[dim * idx[j + k]]), eps);
        A[(size_t)m * i + j + k] = v;
        if (i != j + k) A[(size_t)m * (j + k) + i] = v;
      }
    }
    for (; j < m; j++) {
      double v = orc_phi_scalar(kernel, adist_scalar(dim, xi, &coords[dim * idx[j]]), eps);
      A[(size_t)m * i + j] = v;
      if (i != j) A[(size_t)m * j + i] = v;
    }
  }
}

void orc_assemble(const orc_pu *pu, int kernel, int m, const int *idx, const double *coords, double *A)
{
  assemble(pu, kernel, m, idx, coords, A);
}

/* Lower Cholesky in place (row-major, lower triangle used); left-looking, ascending-k dot
   products.  LAPACK's blocked dpotrf associates differently; results agree to O(kappa*eps). */
static int cholesky(int m, double *A)
{
  int i, j, k;
  for (j = 0; j < m; j++) {
    double d = A[(size_t)m * j + j];
    for (k = 0; k < j; k++) d -= A[(size_t)m * j + k] * A[(size_t)m * j + k];
    if (!(d > 0.0)) return j + 1;
    d = sqrt(d);
    A[(size_t)m * j + j] = d;
    for (i = j + 1; i < m; i++) {
      double s = A[(size_t)m * i + j];
      for (k = 0; k < j; k++) s -= A[(size_t)m * i + k] * A[(size_t)m * j + k];
      A[(size_t)m * i + j] = s / d;
    }
  }
  return 0;
}

static void chol_solve(int m, const double *Lf, double *b)
{
  int i, k;
  for (i = 0; i < m; i++) {
    double s = b[i];
    for (k = 0; k < i; k++) s -= Lf[(size_t)m * i + k] * b[k];
    b[i] = s / Lf[(size_t)m * i + i];
  }
  for (i = m - 1; i >= 0; i--) {
    double s = b[i];
    for (k = i + 1; k < m; k++) s -= Lf[(size_t)m * k + i] * b[k];
    b[i] = s / Lf[(size_t)m * i + i];
  }
}

/* RHS gather of PartitionMatSetRHS (partition_factor.c:57-90) and MatMatSolve. */
static void patch_rhs_solve(int m, const int *idx, const double *Lf, int nfields, const double *values, double *coeffs)
{
  int f, j;
  for (f = 0; f < nfields; f++) {
    double *col = &coeffs[(size_t)f * m];
    for (j = 0; j < m; j++) col[j] = values[(size_t)idx[j] * nfields + f];
    chol_solve(m, Lf, col);
  }
}

int orc_patch_solve(const orc_pu *pu, int kernel, int m, const int *idx, const double *coords,
                    int nfields, const double *values, double *coeffs)
{
  int info;
  double *A;
  if (m == 0) return 0;
  A = (double *)malloc(sizeof(double) * (size_t)m * m);
  assemble(pu, kernel, m, idx, coords, A);
  info = cholesky(m, A);
  if (!info) patch_rhs_solve(m, idx, A, nfields, values, coeffs);
  free(A);
  return info;
}

/* ======================================================================================= */
/* evaluation: PointwiseInterpolation_AVX512 (interpolation_avx512.c:121-291)               */
/* ======================================================================================= */
static inline __attribute__((always_inline)) void
eval_one_k(const orc_pu *pu, const int dim, const int kernel, const double *x, int cell, const double *w,
           const double *restrict xd, const int *blk_start, const int *blk_pts, const int *patch_start,
           const int *patch_pts, const int *patch_setup, double *const *coeffs, int nf, double *restrict rbf_d,
           double *val)
{
  int nen = pu->nen, k, f, nd, i;
  int bs = blk_start[cell], bn = blk_start[cell + 1] - bs;
  const int *bidx = &blk_pts[bs];
  int aligned;
  double eps = pu->eps_r;
  if (bn == 0) return; /* interpolation_avx512.c:184: the value is left untouched */
  aligned = (bn / 8) * 8;
  for (nd = 0; nd < aligned; nd += 8) {
    double r[8];
    for (i = 0; i < 8; i++) {
      int dp = bidx[nd + i];
      double dx = x[0] - xd[dim * dp], dy = x[1] - xd[dim * dp + 1];
      double dz = (dim == 3) ? x[2] - xd[dim * dp + 2] : 0.0;
      r[i] = sqrt((dim == 3) ? fma(dx, dx, fma(dy, dy, dz * dz)) : fma(dx, dx, dy * dy));
    }
    for (i = 0; i < 8; i++) r[i] = phi_lane(kernel, r[i], eps);
    for (i = 0; i < 8; i++) rbf_d[bidx[nd + i]] = r[i];
  }
  for (nd = aligned; nd < bn; nd++) {
    int dp = bidx[nd], d;
    double dist = 0.0;
    for (d = 0; d < dim; d++) { double dx = x[d] - xd[dim * dp + d]; dist += dx * dx; }
    rbf_d[dp] = orc_phi_scalar(kernel, sqrt(dist), eps);
  }
  for (f = 0; f < nf; f++) val[f] = 0.0;
  for (k = 0; k < nen; k++) {
    int node = orc_cell_corner(pu, cell, k);
    int ps = patch_start[node], m = patch_start[node + 1] - ps;
    const int *didx = &patch_pts[ps];
    const double *c = coeffs[node];
    int al;
    double interp[64], acc[8 * 64];
    if (!patch_setup[node] || m == 0 || !c) continue; /* ndata == 0 when the patch is not set up */
    al = (m / 8) * 8;
    /* eight lanes per field; the eight phi values are gathered once for all fields */
    for (f = 0; f < 8 * nf; f++) acc[f] = 0.0;
    for (nd = 0; nd < al; nd += 8) {
      double r[8];
      for (i = 0; i < 8; i++) r[i] = rbf_d[didx[nd + i]];
      for (f = 0; f < nf; f++) {
        const double *cf = &c[(size_t)f * m + nd];
        double *l = &acc[8 * f];
        for (i = 0; i < 8; i++) l[i] = fma(r[i], cf[i], l[i]);
      }
    }
    for (f = 0; f < nf; f++) {
      /* horizontal sum: 512 -> 256 (lo+hi), 256 -> 128 (lo+hi), hadd */
      const double *l = &acc[8 * f];
      double s0 = l[0] + l[4], s1 = l[1] + l[5], s2 = l[2] + l[6], s3 = l[3] + l[7];
      interp[f] = (s0 + s2) + (s1 + s3);
    }
    for (nd = al; nd < m; nd++) {
      double rbf = rbf_d[didx[nd]];
      for (f = 0; f < nf; f++) interp[f] += rbf * c[(size_t)f * m + nd];
    }
    for (f = 0; f < nf; f++) val[f] += interp[f] * w[k];
  }
}

/* eval_one_k with the kernel and the dimension as constants: the reference picks its kernel and
   distance functions once per call (function pointers, interpolation_avx512.c:150-172), so the
   per-element kernel switch of phi_lane is hoisted out of the loops here too. */
static void eval_one(const orc_pu *pu, int kernel, const double *x, int cell, const double *w,
                     const double *xd, const int *blk_start, const int *blk_pts, const int *patch_start,
                     const int *patch_pts, const int *patch_setup, double *const *coeffs, int nf,
                     double *rbf_d, double *val)
{
  if (nf < 1 || nf > 64) return; /* nothing to evaluate / per-field scratch of eval_one_k */
#define ORC_EVAL_K(D, K) eval_one_k(pu, D, K, x, cell, w, xd, blk_start, blk_pts, patch_start, patch_pts, \
                                    patch_setup, coeffs, nf, rbf_d, val)
  if (pu->dim == 3) {
    switch (kernel) {
    case ORC_KERNEL_WENDLAND_C2: ORC_EVAL_K(3, ORC_KERNEL_WENDLAND_C2); return;
    case ORC_KERNEL_GAUSSIAN: ORC_EVAL_K(3, ORC_KERNEL_GAUSSIAN); return;
    default: ORC_EVAL_K(3, kernel); return;
    }
  }
  switch (kernel) {
  case ORC_KERNEL_WENDLAND_C2: ORC_EVAL_K(2, ORC_KERNEL_WENDLAND_C2); return;
  case ORC_KERNEL_GAUSSIAN: ORC_EVAL_K(2, ORC_KERNEL_GAUSSIAN); return;
  default: ORC_EVAL_K(2, kernel); return;
  }
#undef ORC_EVAL_K
}

static void eval_all(const orc_pu *pu, int kernel, int np, const double *xp, const int *cellid, const int *alive,
                     const double *weights, const double *xd, const int *blk_start, const int *blk_pts,
                     const int *patch_start, const int *patch_pts, const int *patch_setup, double *const *coeffs,
                     int nf, double *values, double *rbf_d)
{
  int p;
  for (p = 0; p < np; p++) {
    if (alive && !alive[p]) continue;
    if (cellid[p] < 0) continue;
    eval_one(pu, kernel, &xp[pu->dim * p], cellid[p], &weights[pu->nen * p], xd, blk_start, blk_pts,
             patch_start, patch_pts, patch_setup, coeffs, nf, rbf_d, &values[(size_t)nf * p]);
  }
}

void orc_eval(const orc_pu *pu, int kernel, int np, const double *xp, const int *cellid, const int *alive,
              const double *weights, const double *xd, const int *blk_start, const int *blk_pts,
              const int *patch_start, const int *patch_pts, const int *patch_setup, double *const *coeffs,
              int nf, double *values)
{
  int p;
  long nd = 0;
  double *rbf_d;
  /* scratch rbf_d is sized by the largest data index referenced by the blocks */
  for (p = 0; p < blk_start[pu->ncells]; p++) if (blk_pts[p] + 1 > nd) nd = blk_pts[p] + 1;
  rbf_d = (double *)calloc((size_t)nd + 1, sizeof(double));
  for (p = 0; p < np; p++) {
    if (alive && !alive[p]) continue;
    if (cellid[p] < 0) continue;
    eval_one(pu, kernel, &xp[pu->dim * p], cellid[p], &weights[pu->nen * p], xd, blk_start, blk_pts,
             patch_start, patch_pts, patch_setup, coeffs, nf, rbf_d, &values[(size_t)nf * p]);
  }
  free(rbf_d);
}

/* ======================================================================================= */
/* reference-API emulation                                                                  */
/* ======================================================================================= */
struct orc_ctx {
  orc_config cfg;
  orc_pu pu;
  /* data swarm (swarm_data.c:51-88) */
  int nd, nd_cap;
  double *xd, *fd;
  int64_t *pid_d;
  int *cell_d, *cell_start, *cell_pts, *blk_start, *blk_pts;
  int data_binned;
  /* patches (partition.c) */
  int *patch_setup, *patch_solved, *patch_start, *patch_pts; /* membership captured at setup */
  long patch_len;
  int **patch_idx;       /* per-patch data_idx, owned when set up */
  int *patch_m;
  double **coeffs;       /* per-patch column-major coefficients */
  double **factor;       /* per-patch Cholesky factor kept by A_FACTOR / A_KSP */
  /* interpolation swarm (swarm_interp.c:72-118) */
  int np, np_cap;
  double *xp, *fields, *vel, *weights, *x0, *vadv[7];
  int64_t *pid_p;
  int *cell_p, *alive;
  /* advection */
  double dt;             /* AdvectionCtx dt; DOPRI writes its adapted step here */
  double dopri_error;
  int nsteps;
  /* per-particle Dormand-Prince (extension): time reached, next step, step of the sweep */
  double *tp, *hp, *hcur;
  int *act, *clamped;
  long long pp_accepted;
  orc_velocity_fn vfn;
  orc_velocity_batch_fn vfn_batch;
  void *vuser;
  orc_step_reduce_fn reduce;
  void *ruser;
};

static void *xrealloc(void *p, size_t n) { void *q = realloc(p, n ? n : 1); return q; }

orc_ctx *orc_create(const orc_config *cfg)
{
  orc_ctx *c;
  int n;
  if (cfg->dim != 2 && cfg->dim != 3) return NULL; /* cell_info.c:312-324 */
  if (cfg->nfields < 0 || cfg->nfields > 64) return NULL; /* per-field scratch of the evaluation */
  for (n = 0; n < cfg->dim; n++) if (cfg->n[n] < 2) return NULL;
  c = (orc_ctx *)calloc(1, sizeof(*c));
  c->cfg = *cfg;
  orc_pu_setup(&c->pu, cfg);
  c->patch_setup = (int *)calloc((size_t)c->pu.nnodes, sizeof(int));
  c->patch_solved = (int *)calloc((size_t)c->pu.nnodes, sizeof(int));
  c->patch_idx = (int **)calloc((size_t)c->pu.nnodes, sizeof(int *));
  c->patch_m = (int *)calloc((size_t)c->pu.nnodes, sizeof(int));
  c->coeffs = (double **)calloc((size_t)c->pu.nnodes, sizeof(double *));
  c->factor = (double **)calloc((size_t)c->pu.nnodes, sizeof(double *));
  c->patch_start = (int *)calloc((size_t)c->pu.nnodes + 1, sizeof(int));
  c->cell_start = (int *)calloc((size_t)c->pu.ncells + 1, sizeof(int));
  c->blk_start = (int *)calloc((size_t)c->pu.ncells + 1, sizeof(int));
  c->dt = cfg->dt;
  c->dopri_error = ORC_MAX_REAL;
  return c;
}

static void patch_reset_one(orc_ctx *c, int n)
{
  /* PartitionReset_SinglePartition, partition.c:235-250 */
  c->patch_solved[n] = 0;
  c->patch_setup[n] = 0;
  free(c->patch_idx[n]); c->patch_idx[n] = NULL; c->patch_m[n] = 0;
  free(c->coeffs[n]); c->coeffs[n] = NULL;
  free(c->factor[n]); c->factor[n] = NULL;
}

void orc_destroy(orc_ctx *c)
{
  int n, s;
  if (!c) return;
  for (n = 0; n < c->pu.nnodes; n++) patch_reset_one(c, n);
  free(c->patch_setup); free(c->patch_solved); free(c->patch_idx); free(c->patch_m);
  free(c->coeffs); free(c->factor); free(c->patch_start); free(c->patch_pts);
  free(c->xd); free(c->fd); free(c->pid_d); free(c->cell_d); free(c->cell_start); free(c->cell_pts);
  free(c->blk_start); free(c->blk_pts);
  free(c->xp); free(c->fields); free(c->vel); free(c->weights); free(c->x0);
  for (s = 0; s < 7; s++) free(c->vadv[s]);
  free(c->pid_p); free(c->cell_p); free(c->alive);
  free(c->tp); free(c->hp); free(c->hcur); free(c->act); free(c->clamped);
  free(c);
}

/* SwarmFieldAssignUniqueIndex (swarm_utils.c:37-73) on one rank: pid = max(existing) + 1 + p,
   where "existing" are the values the resized swarm still holds (DMSwarmSetLocalSizes keeps the
   first min(old,new) entries and zeroes the rest). */
static void assign_pid(int64_t *pid, int old_n, int new_n)
{
  int p;
  int64_t mx = 0;
  for (p = 0; p < new_n; p++) {
    int64_t v = (p < old_n) ? pid[p] : 0;
    if (v > mx) mx = v;
  }
  mx += 1;
  for (p = 0; p < new_n; p++) pid[p] = mx + p;
}

static int check_inside_box(const orc_pu *pu, int n, const double *coords)
{
  /* DMSwarmAssignRankFromDMDA (swarm_utils.c:854-871): a point outside the bounding box of the
     (single-rank) DMDA is an error. */
  int p, d;
  for (p = 0; p < n; p++)
    for (d = 0; d < pu->dim; d++) {
      double x = coords[pu->dim * p + d];
      if (x < pu->O[d] || x > pu->L[d]) return ORC_ERR_ARG_WRONG;
    }
  return 0;
}

int orc_fill_swarm(orc_ctx *c, int is_data, int n, const double *coords, const double *values,
                   const int64_t *pidx)
{
  int dim = c->pu.dim, F = c->cfg.nfields, nen = c->pu.nen, p, s;
  if (n < 0) return ORC_ERR_ARG_OUTOFRANGE;
  if (n > 0 && !coords) return ORC_ERR_ARG_NULL;
  if (check_inside_box(&c->pu, n, coords)) return ORC_ERR_ARG_WRONG;
  if (is_data) {
    int old = c->nd;
    c->xd = (double *)xrealloc(c->xd, sizeof(double) * (size_t)n * dim);
    c->fd = (double *)xrealloc(c->fd, sizeof(double) * (size_t)n * (F ? F : 1));
    c->pid_d = (int64_t *)xrealloc(c->pid_d, sizeof(int64_t) * (size_t)(n ? n : 1));
    for (p = old; p < n; p++) c->pid_d[p] = 0;
    if (n > old) memset(&c->fd[(size_t)old * F], 0, sizeof(double) * (size_t)(n - old) * F);
    c->cell_d = (int *)xrealloc(c->cell_d, sizeof(int) * (size_t)(n ? n : 1));
    c->cell_pts = (int *)xrealloc(c->cell_pts, sizeof(int) * (size_t)(n ? n : 1));
    if (n) memcpy(c->xd, coords, sizeof(double) * (size_t)n * dim);
    if (values && n) memcpy(c->fd, values, sizeof(double) * (size_t)n * F);
    if (pidx) { if (n) memcpy(c->pid_d, pidx, sizeof(int64_t) * (size_t)n); }
    else assign_pid(c->pid_d, old, n);
    c->nd = n;
    /* DMSwarmPICSetCellId + CellInfoSetUp (interface_utils.c:140-165) */
    orc_locate(&c->pu, n, c->xd, c->cell_d);
    orc_cell_csr(&c->pu, n, c->cell_d, c->cell_start, c->cell_pts);
    {
      long bl = orc_block_csr(&c->pu, c->cell_start, c->cell_pts, NULL, NULL);
      c->blk_pts = (int *)xrealloc(c->blk_pts, sizeof(int) * (size_t)(bl ? bl : 1));
      orc_block_csr(&c->pu, c->cell_start, c->cell_pts, c->blk_start, c->blk_pts);
    }
    c->data_binned = 1;
    return 0;
  }
  {
    int old = c->np;
    c->xp = (double *)xrealloc(c->xp, sizeof(double) * (size_t)n * dim);
    c->fields = (double *)xrealloc(c->fields, sizeof(double) * (size_t)n * (F ? F : 1));
    c->vel = (double *)xrealloc(c->vel, sizeof(double) * (size_t)n * dim);
    c->weights = (double *)xrealloc(c->weights, sizeof(double) * (size_t)n * nen);
    c->x0 = (double *)xrealloc(c->x0, sizeof(double) * (size_t)n * dim);
    for (s = 0; s < 7; s++) c->vadv[s] = (double *)xrealloc(c->vadv[s], sizeof(double) * (size_t)n * dim);
    c->pid_p = (int64_t *)xrealloc(c->pid_p, sizeof(int64_t) * (size_t)(n ? n : 1));
    c->cell_p = (int *)xrealloc(c->cell_p, sizeof(int) * (size_t)(n ? n : 1));
    c->alive = (int *)xrealloc(c->alive, sizeof(int) * (size_t)(n ? n : 1));
    c->tp = (double *)xrealloc(c->tp, sizeof(double) * (size_t)(n ? n : 1));
    c->hp = (double *)xrealloc(c->hp, sizeof(double) * (size_t)(n ? n : 1));
    c->hcur = (double *)xrealloc(c->hcur, sizeof(double) * (size_t)(n ? n : 1));
    c->act = (int *)xrealloc(c->act, sizeof(int) * (size_t)(n ? n : 1));
    c->clamped = (int *)xrealloc(c->clamped, sizeof(int) * (size_t)(n ? n : 1));
    for (p = 0; p < n; p++) c->hp[p] = 0.0; /* a new swarm starts from the context step */
    for (p = old; p < n; p++) c->pid_p[p] = 0;
    if (n > old) {
      memset(&c->fields[(size_t)old * F], 0, sizeof(double) * (size_t)(n - old) * F);
      memset(&c->vel[(size_t)old * dim], 0, sizeof(double) * (size_t)(n - old) * dim);
      memset(&c->weights[(size_t)old * nen], 0, sizeof(double) * (size_t)(n - old) * nen);
    }
    if (n) memcpy(c->xp, coords, sizeof(double) * (size_t)n * dim);
    if (values && n) memcpy(c->fields, values, sizeof(double) * (size_t)n * F);
    if (pidx) { if (n) memcpy(c->pid_p, pidx, sizeof(int64_t) * (size_t)n); }
    else assign_pid(c->pid_p, old, n);
    c->np = n;
    for (p = 0; p < n; p++) c->alive[p] = 1;
    /* FillInterpSwarm (interface_utils.c:118-138): cell ids + weights */
    orc_locate(&c->pu, n, c->xp, c->cell_p);
    orc_weights(&c->pu, n, c->xp, c->cell_p, c->alive, c->weights);
    return 0;
  }
}

/* Lazy patch set-up and solve (LagRBF_PartitionsSetUp, partition.c:417-478). */
/* LagRBF_PartitionsSetUp for one patch node (partition.c:417-478): set up (membership, assembly,
   factor) and solve when not done yet. */
static int setup_node(orc_ctx *c, int node)
{
  int F = c->cfg.nfields;
  if (!c->patch_setup[node]) {
    /* PartitionSetUp_SinglePartition: membership from the current data-swarm sort */
    long len = orc_patch_csr(&c->pu, c->cell_start, c->cell_pts, NULL, NULL);
    int m, info;
    if (len != c->patch_len || !c->patch_pts) {
      c->patch_pts = (int *)xrealloc(c->patch_pts, sizeof(int) * (size_t)(len ? len : 1));
      c->patch_len = len;
    }
    orc_patch_csr(&c->pu, c->cell_start, c->cell_pts, c->patch_start, c->patch_pts);
    m = c->patch_start[node + 1] - c->patch_start[node];
    c->patch_idx[node] = (int *)malloc(sizeof(int) * (size_t)(m ? m : 1));
    if (m) memcpy(c->patch_idx[node], &c->patch_pts[c->patch_start[node]], sizeof(int) * (size_t)m);
    c->patch_m[node] = m;
    c->coeffs[node] = (double *)calloc((size_t)(m ? m : 1) * (F ? F : 1), sizeof(double));
    if (m) {
      double *A = (double *)malloc(sizeof(double) * (size_t)m * m);
      assemble(&c->pu, c->cfg.kernel, m, c->patch_idx[node], c->xd, A);
      info = cholesky(m, A);
      if (info) { free(A); return ORC_ERR_MAT_CH_ZRPVT; }
      c->factor[node] = A;
    }
    c->patch_setup[node] = 1;
  }
  if (!c->patch_solved[node]) {
    /* PartitionSolveInterpolationCoefficients_SinglePartition, partition_solve.c:97-113 */
    int m = c->patch_m[node];
    if (m > 0) {
      patch_rhs_solve(m, c->patch_idx[node], c->factor[node], F, c->fd, c->coeffs[node]);
      if (c->cfg.solve_method == ORC_A_KSP_ASMB || c->cfg.solve_method == ORC_A_FACTOR) {
        /* the assembled/factored matrix is released after the solve; A_FACTOR reloads its
           factor from disk on the next solve, which keeping it here reproduces */
        if (c->cfg.solve_method == ORC_A_KSP_ASMB) { free(c->factor[node]); c->factor[node] = NULL; }
      }
      c->patch_solved[node] = 1;
    }
  }
  return 0;
}

static int partitions_setup(orc_ctx *c)
{
  int p, k, node, err;
  if (c->cfg.setup_all) { /* extension: every patch, independent of where the particles are */
    for (node = 0; node < c->pu.nnodes; node++)
      if ((err = setup_node(c, node))) return err;
    return 0;
  }
  for (p = 0; p < c->np; p++) {
    if (!c->alive[p] || c->cell_p[p] < 0) continue;
    for (k = 0; k < c->pu.nen; k++)
      if ((err = setup_node(c, orc_cell_corner(&c->pu, c->cell_p[p], k)))) return err;
  }
  return 0;
}

/* Evaluation over all live particles of the interpolation swarm. */
static void rbf_interpolation(orc_ctx *c, int nf, double *values)
{
  int node;
  long len = 0;
  int *ps, *pp, *setup;
  double **cf;
  /* per-patch arrays captured at set-up time */
  ps = (int *)malloc(sizeof(int) * ((size_t)c->pu.nnodes + 1));
  setup = (int *)malloc(sizeof(int) * (size_t)c->pu.nnodes);
  cf = (double **)malloc(sizeof(double *) * (size_t)c->pu.nnodes);
  for (node = 0; node < c->pu.nnodes; node++) { ps[node] = (int)len; len += c->patch_setup[node] ? c->patch_m[node] : 0; }
  ps[c->pu.nnodes] = (int)len;
  pp = (int *)malloc(sizeof(int) * (size_t)(len ? len : 1));
  for (node = 0; node < c->pu.nnodes; node++) {
    setup[node] = c->patch_setup[node];
    cf[node] = c->patch_setup[node] ? c->coeffs[node] : NULL;
    if (c->patch_setup[node] && c->patch_m[node])
      memcpy(&pp[ps[node]], c->patch_idx[node], sizeof(int) * (size_t)c->patch_m[node]);
  }
  {
    double *rbf_d = (double *)calloc((size_t)c->nd + 1, sizeof(double));
    eval_all(&c->pu, c->cfg.kernel, c->np, c->xp, c->cell_p, c->alive, c->weights, c->xd, c->blk_start,
             c->blk_pts, ps, pp, setup, cf, nf, values, rbf_d);
    free(rbf_d);
  }
  free(ps); free(pp); free(setup); free(cf);
}

int orc_interpolation(orc_ctx *c)
{
  int err;
  if (!c->data_binned) return ORC_ERR_ARG_NULL;
  err = partitions_setup(c);
  if (err) return err;
  rbf_interpolation(c, c->cfg.nfields, c->fields);
  return 0;
}

int orc_output(orc_ctx *c, int is_data, int nglobal, double *coords, double *fields, int64_t *pidx,
               const char *fieldname)
{
  /* Interface_Output_Allreduce / AssembleArray_Allreduce (interface_utils.c:188-339) */
  int dim = c->pu.dim, n = is_data ? c->nd : c->np, p, f, nf = 0;
  const int64_t *pid = is_data ? c->pid_d : c->pid_p;
  const double *src = NULL;
  if (fields) {
    if (!fieldname || strcmp(fieldname, "fields") == 0) { src = is_data ? c->fd : c->fields; nf = c->cfg.nfields; }
    else if (!is_data && strcmp(fieldname, "velocity") == 0) { src = c->vel; nf = dim; }
    else if (!is_data && strcmp(fieldname, "weights") == 0) { src = c->weights; nf = c->pu.nen; }
    else return ORC_ERR_ARG_WRONG;
  }
  if (coords) memset(coords, 0, sizeof(double) * (size_t)nglobal * dim);
  if (fields) memset(fields, 0, sizeof(double) * (size_t)nglobal * nf);
  if (pidx) memset(pidx, 0, sizeof(int64_t) * (size_t)nglobal);
  for (p = 0; p < n; p++) {
    int64_t g;
    if (!is_data && !c->alive[p]) continue; /* removed by migration */
    g = pid[p] - 1;
    if (g < 0 || g >= nglobal) return ORC_ERR_ARG_OUTOFRANGE;
    if (coords) for (f = 0; f < dim; f++) coords[g * dim + f] = (is_data ? c->xd : c->xp)[(size_t)p * dim + f];
    if (fields) for (f = 0; f < nf; f++) fields[g * nf + f] = src[(size_t)p * nf + f];
    if (pidx) pidx[g] = pid[p];
  }
  return 0;
}

int orc_reset_coefficients(orc_ctx *c)
{
  int n;
  for (n = 0; n < c->pu.nnodes; n++) {
    if (c->cfg.solve_method == ORC_A_KSP_ASMB) patch_reset_one(c, n);
    else c->patch_solved[n] = 0;
  }
  return 0;
}

/* --------------------------------- advection ---------------------------------------- */
/* AdvectionProjectOntoSphereBoundary_Pointwise (advection.c:472-491) */
static void project_sphere(double *x, int dim, double rmin, double rmax)
{
  int d;
  double pos = 0.0, normal[3];
  for (d = 0; d < dim; d++) pos += x[d] * x[d];
  if (pos < rmax * rmax && pos > rmin * rmin) return;
  pos = sqrt(pos);
  for (d = 0; d < dim; d++) normal[d] = x[d] / pos;
  if (pos > rmax) for (d = 0; d < dim; d++) x[d] = rmax * normal[d];
  else for (d = 0; d < dim; d++) x[d] = rmin * normal[d];
}

/* DMSwarmMigrate on one rank: relocate, drop particles that left the domain; then
   SwarmInterpSetWeights. */
static void migrate_and_weights(orc_ctx *c)
{
  int p;
  orc_locate(&c->pu, c->np, c->xp, c->cell_p);
  for (p = 0; p < c->np; p++) if (c->alive[p] && c->cell_p[p] < 0) c->alive[p] = 0;
  orc_weights(&c->pu, c->np, c->xp, c->cell_p, c->alive, c->weights);
}

static int evaluate_velocity(orc_ctx *c)
{
  /* AdvectionEvaluateVelocity (advection.c:391-414) */
  int dim = c->pu.dim, p;
  if (c->vfn_batch || c->vfn) {
    /* analytical: the callback sees the live particles packed contiguously */
    int nl = 0, q = 0, err = 0;
    double *xc, *vc;
    for (p = 0; p < c->np; p++) nl += c->alive[p];
    xc = (double *)malloc(sizeof(double) * (size_t)(nl ? nl : 1) * dim);
    vc = (double *)malloc(sizeof(double) * (size_t)(nl ? nl : 1) * dim);
    for (p = 0; p < c->np; p++) if (c->alive[p]) { memcpy(&xc[(size_t)q * dim], &c->xp[(size_t)p * dim], sizeof(double) * dim); q++; }
    memset(vc, 0, sizeof(double) * (size_t)(nl ? nl : 1) * dim);
    if (c->vfn_batch) err = c->vfn_batch(nl, dim, xc, vc, c->vuser);
    else for (q = 0; q < nl && !err; q++) err = c->vfn(&xc[(size_t)q * dim], &vc[(size_t)q * dim], c->vuser);
    q = 0;
    for (p = 0; p < c->np; p++) if (c->alive[p]) { memcpy(&c->vel[(size_t)p * dim], &vc[(size_t)q * dim], sizeof(double) * dim); q++; }
    free(xc); free(vc);
    return err;
  }
  rbf_interpolation(c, dim, c->vel);
  return 0;
}

static void copy_fields_to_velocity(orc_ctx *c)
{
  /* AdvectionCopyVelocityField (advection.c:298-316) */
  int p, d, dim = c->pu.dim, F = c->cfg.nfields;
  for (p = 0; p < c->np; p++)
    for (d = 0; d < dim; d++) c->vel[(size_t)p * dim + d] = (d < F) ? c->fields[(size_t)p * F + d] : 0.0;
}

static int initialize_timestep_velocity(orc_ctx *c)
{
  /* AdvectionInitializeTimestepVelocity (advection.c:353-373) */
  if (c->vfn_batch || c->vfn) return evaluate_velocity(c);
  copy_fields_to_velocity(c);
  return 0;
}

static void euler(orc_ctx *c, double *x, const double *x0, const double *v, double dt)
{
  /* AdvectionExplicit_Scalar (advection.c:36-57) */
  int p, d, dim = c->pu.dim;
  for (p = 0; p < c->np; p++) {
    if (!c->alive[p]) continue;
    for (d = 0; d < dim; d++) x[(size_t)p * dim + d] = x0[(size_t)p * dim + d] + dt * v[(size_t)p * dim + d];
  }
}

static int rk1(orc_ctx *c)
{
  /* runge_kutta_1.c:37-75 */
  int dim = c->pu.dim;
  memcpy(c->x0, c->xp, sizeof(double) * (size_t)c->np * dim);
  euler(c, c->xp, c->x0, c->vel, c->dt);
  migrate_and_weights(c);
  return 0;
}

static int rk2(orc_ctx *c)
{
  /* runge_kutta_2.c:38-91 */
  int dim = c->pu.dim, err;
  memcpy(c->x0, c->xp, sizeof(double) * (size_t)c->np * dim);
  euler(c, c->xp, c->x0, c->vel, 0.5 * c->dt);
  migrate_and_weights(c);
  if ((err = evaluate_velocity(c))) return err;
  euler(c, c->xp, c->x0, c->vel, c->dt);
  migrate_and_weights(c);
  return 0;
}

static void set_initial_values(orc_ctx *c)
{
  /* AdvectionSetInitialValues (advection.c:248-278) */
  int dim = c->pu.dim;
  memcpy(c->x0, c->xp, sizeof(double) * (size_t)c->np * dim);
  memcpy(c->vadv[0], c->vel, sizeof(double) * (size_t)c->np * dim);
}

static int rk4(orc_ctx *c)
{
  /* runge_kutta_4.c:45-156 */
  static const double coef[3] = {0.5, 0.5, 1.0};
  static const double wts[4] = {1.0, 2.0, 2.0, 1.0};
  int dim = c->pu.dim, s, p, d, err;
  double dt = c->dt;
  set_initial_values(c);
  for (s = 0; s < 3; s++) {
    memcpy(c->vel, c->vadv[s], sizeof(double) * (size_t)c->np * dim);
    euler(c, c->xp, c->x0, c->vel, coef[s] * dt);
    for (p = 0; p < c->np; p++) if (c->alive[p]) project_sphere(&c->xp[(size_t)p * dim], dim, c->cfg.rmin, c->cfg.rmax);
    migrate_and_weights(c);
    if ((err = evaluate_velocity(c))) return err;
    memcpy(c->vadv[s + 1], c->vel, sizeof(double) * (size_t)c->np * dim);
  }
  for (p = 0; p < c->np; p++) {
    double sum[3] = {0.0, 0.0, 0.0};
    if (!c->alive[p]) continue;
    for (d = 0; d < dim; d++) {
      for (s = 0; s < 4; s++) sum[d] += wts[s] * c->vadv[s][(size_t)p * dim + d];
      c->xp[(size_t)p * dim + d] = c->x0[(size_t)p * dim + d] + dt / 6.0 * sum[d];
      /* runge_kutta_4.c:140: projection inside the per-component loop */
      project_sphere(&c->xp[(size_t)p * dim], dim, c->cfg.rmin, c->cfg.rmax);
    }
  }
  migrate_and_weights(c);
  return 0;
}

static const double DP_A[6][6] = {
  {1.0 / 5.0, 0, 0, 0, 0, 0},
  {3.0 / 40.0, 9.0 / 40.0, 0, 0, 0, 0},
  {44.0 / 45.0, -56.0 / 15.0, 32.0 / 9.0, 0, 0, 0},
  {19372.0 / 6561.0, -25360.0 / 2187.0, 64448.0 / 6561.0, -212.0 / 729.0, 0, 0},
  {9017.0 / 3168.0, -355.0 / 33.0, 46732.0 / 5247.0, 49.0 / 176.0, -5103.0 / 18656.0, 0},
  {35.0 / 384.0, 0, 500.0 / 1113.0, 125.0 / 192.0, -2187.0 / 6784.0, 11.0 / 84.0}};
static const double DP_E[7] = {5179.0 / 57600.0, 0, 7571.0 / 16695.0, 393.0 / 640.0, -92097.0 / 339200.0,
                               187.0 / 2100.0, 1.0 / 40.0};

static int dopri(orc_ctx *c)
{
  /* dormand_prince.c:216-310 (Butcher rows :224-231), error :37-102, adaptive dt :179-214 */
  int dim = c->pu.dim, s, j, p, d, err;
  double dt = c->dt, max_err, fac, fac_min, fac_max, dt_new;
  set_initial_values(c);
  for (s = 0; s < 6; s++) {
    int stage = s + 1;
    for (p = 0; p < c->np; p++) {
      if (!c->alive[p]) { for (d = 0; d < dim; d++) c->vel[(size_t)p * dim + d] = 0.0; continue; }
      for (d = 0; d < dim; d++) c->vel[(size_t)p * dim + d] = 0.0;
      for (j = 0; j < stage; j++)
        for (d = 0; d < dim; d++) c->vel[(size_t)p * dim + d] += DP_A[s][j] * c->vadv[j][(size_t)p * dim + d];
      for (d = 0; d < dim; d++) c->xp[(size_t)p * dim + d] = c->x0[(size_t)p * dim + d] + dt * c->vel[(size_t)p * dim + d];
      project_sphere(&c->xp[(size_t)p * dim], dim, c->cfg.rmin, c->cfg.rmax);
    }
    migrate_and_weights(c);
    if ((err = evaluate_velocity(c))) return err;
    memcpy(c->vadv[stage], c->vel, sizeof(double) * (size_t)c->np * dim);
  }
  max_err = -ORC_MAX_REAL; /* PETSC_MIN_REAL */
  for (p = 0; p < c->np; p++) {
    double vlow[3] = {0.0, 0.0, 0.0}, E = 0.0;
    if (!c->alive[p]) continue;
    for (s = 0; s < 7; s++)
      for (d = 0; d < dim; d++) vlow[d] += DP_E[s] * c->vadv[s][(size_t)p * dim + d];
    for (d = 0; d < dim; d++) {
      double x0 = c->x0[(size_t)p * dim + d], x = c->xp[(size_t)p * dim + d];
      double mv = ORC_MAX(fabs(x0), fabs(x));
      double tol = c->cfg.dopri_atol + c->cfg.dopri_rtol * mv;
      double xl = x0 + dt * vlow[d];
      double e = x - xl;
      E += (e * e) / (tol * tol);
    }
    E = sqrt(1.0 / dim * E);
    max_err = ORC_MAX(max_err, E);
  }
  if (c->reduce) { /* global maximum of the error over the ranks (dormand_prince.c:93) */
    double v[2] = {-ORC_MAX_REAL, max_err};
    if ((err = c->reduce(v, 2, c->ruser))) return err;
    max_err = v[1];
  }
  c->dopri_error = max_err;
  migrate_and_weights(c);
  fac = c->cfg.dopri_dt_fac;
  fac_min = c->cfg.dopri_dt_fac_min;
  fac_max = (max_err <= 1.0) ? c->cfg.dopri_dt_fac_max : 1.0;
  dt_new = dt * ORC_MIN(fac_max, ORC_MAX(fac_min, fac * pow(1.0 / max_err, 1.0 / 5.0)));
  c->dt = dt_new;
  return 0;
}

/* Per-particle adaptive Dormand-Prince, one sweep (an extension; the reference's scheme above takes
   one global step from the global maximum error and always accepts it).  Every live particle p
   short of t_next attempts a step h_p = min(hp_p, its own CFL step cfl r / (|v_p| + 1e-16),
   t_next - tp_p) with the same stages and error norm E_p as dormand_prince.c:37-102, 216-310; the
   step is accepted when E_p <= 1 (or when h_p has fallen below hmin, so that no particle stalls),
   else the particle returns to x0; either way hp_p = h_p min(fac_max', max(fac_min, fac E_p^-1/5))
   with fac_max' = fac_max after an accepted step and 1 after a rejected one (dormand_prince.c:
   179-214 per particle).  Particles that are done keep their position; their stage velocities are
   evaluated but unused. */
static int dopri_pp_sweep(orc_ctx *c, double t_next, double hmin)
{
  int dim = c->pu.dim, s, j, p, d, err;
  const double radius = 1.0 / c->pu.eps_w;
  for (p = 0; p < c->np; p++) {
    double nv = 0.0, h, cfl;
    c->act[p] = c->alive[p] && c->tp[p] < t_next;
    c->clamped[p] = 0;
    c->hcur[p] = 0.0;
    if (!c->act[p]) continue;
    for (d = 0; d < dim; d++) nv += c->vel[(size_t)p * dim + d] * c->vel[(size_t)p * dim + d];
    cfl = c->cfg.cfl_fac * radius / (sqrt(nv) + 1e-16);
    h = ORC_MIN(c->hp[p], cfl);
    if (c->tp[p] + h >= t_next) { h = t_next - c->tp[p]; c->clamped[p] = 1; }
    c->hcur[p] = h;
  }
  set_initial_values(c);
  for (s = 0; s < 6; s++) {
    int stage = s + 1;
    for (p = 0; p < c->np; p++) {
      if (!c->alive[p] || !c->act[p]) continue;
      for (d = 0; d < dim; d++) c->vel[(size_t)p * dim + d] = 0.0;
      for (j = 0; j < stage; j++)
        for (d = 0; d < dim; d++) c->vel[(size_t)p * dim + d] += DP_A[s][j] * c->vadv[j][(size_t)p * dim + d];
      for (d = 0; d < dim; d++)
        c->xp[(size_t)p * dim + d] = c->x0[(size_t)p * dim + d] + c->hcur[p] * c->vel[(size_t)p * dim + d];
      project_sphere(&c->xp[(size_t)p * dim], dim, c->cfg.rmin, c->cfg.rmax);
    }
    migrate_and_weights(c);
    if ((err = evaluate_velocity(c))) return err;
    memcpy(c->vadv[stage], c->vel, sizeof(double) * (size_t)c->np * dim);
  }
  for (p = 0; p < c->np; p++) {
    double vlow[3] = {0.0, 0.0, 0.0}, E = 0.0, h = c->hcur[p], fmax, f;
    int acc;
    if (!c->act[p] || !c->alive[p]) continue;
    for (s = 0; s < 7; s++)
      for (d = 0; d < dim; d++) vlow[d] += DP_E[s] * c->vadv[s][(size_t)p * dim + d];
    for (d = 0; d < dim; d++) {
      double x0 = c->x0[(size_t)p * dim + d], x = c->xp[(size_t)p * dim + d];
      double mv = ORC_MAX(fabs(x0), fabs(x));
      double tol = c->cfg.dopri_atol + c->cfg.dopri_rtol * mv;
      double e = x - (x0 + h * vlow[d]);
      E += (e * e) / (tol * tol);
    }
    E = sqrt(1.0 / dim * E);
    acc = (E <= 1.0) || (h < hmin);
    if (acc) {
      c->tp[p] = c->clamped[p] ? t_next : c->tp[p] + h;
      c->pp_accepted++;
    } else {
      for (d = 0; d < dim; d++) c->xp[(size_t)p * dim + d] = c->x0[(size_t)p * dim + d];
    }
    fmax = (E <= 1.0) ? c->cfg.dopri_dt_fac_max : 1.0;
    f = ORC_MIN(fmax, ORC_MAX(c->cfg.dopri_dt_fac_min, c->cfg.dopri_dt_fac * pow(1.0 / E, 1.0 / 5.0)));
    c->hp[p] = h * f;
  }
  migrate_and_weights(c);
  return 0;
}

long long orc_get_accepted(orc_ctx *c) { return c->pp_accepted; }

static int advect_swarm(orc_ctx *c)
{
  switch (c->cfg.scheme) {
  case ORC_RK1: return rk1(c);
  case ORC_RK2: return rk2(c);
  case ORC_RK4: return rk4(c);
  case ORC_DOPRI: return dopri(c);
  default: return ORC_ERR_ARG_OUTOFRANGE;
  }
}

static double cfl_dt(orc_ctx *c)
{
  /* AdvectionComputeTimestep_CFL (advection.c:430-470) */
  int p, d, dim = c->pu.dim;
  double radius = 1.0 / c->pu.eps_w, dt = ORC_MAX_REAL;
  for (p = 0; p < c->np; p++) {
    double nv = 0.0, dl;
    if (!c->alive[p]) continue;
    for (d = 0; d < dim; d++) nv += c->vel[(size_t)p * dim + d] * c->vel[(size_t)p * dim + d];
    nv = sqrt(nv);
    dl = c->cfg.cfl_fac * radius / (nv + 1e-16);
    dt = ORC_MIN(dt, dl);
  }
  return dt;
}

static int advection_loop(orc_ctx *c, double t, double t_next, int interpolated, int keep)
{
  /* InternalForwardAdvectionLoop (time_loop.c:39-100) / ForwardAnalyticalAdvection (:176-221) */
  int err;
  if ((err = initialize_timestep_velocity(c))) return err;
  if (c->cfg.scheme == ORC_DOPRI && c->cfg.dopri_per_particle) {
    const double hmin = 1e-10 * (t_next - t);
    int p, left = 1;
    for (p = 0; p < c->np; p++) {
      c->tp[p] = t;
      if (!(c->hp[p] > 0.0)) c->hp[p] = c->dt;
    }
    while (left) {
      if ((err = dopri_pp_sweep(c, t_next, hmin))) return err;
      if (interpolated) {
        if ((err = partitions_setup(c))) return err;
        rbf_interpolation(c, c->cfg.nfields, c->fields);
      }
      if ((err = initialize_timestep_velocity(c))) return err;
      c->nsteps++;
      left = 0;
      for (p = 0; p < c->np; p++) left |= c->alive[p] && c->tp[p] < t_next;
    }
  }
  while (t < t_next && !(c->cfg.scheme == ORC_DOPRI && c->cfg.dopri_per_particle)) {
    double dt;
    if (c->cfg.scheme == ORC_DOPRI) {
      double dt_cfl = cfl_dt(c);
      if (c->reduce) { /* global minimum of the CFL step over the ranks (advection.c:466) */
        double v[2] = {-dt_cfl, -ORC_MAX_REAL};
        if ((err = c->reduce(v, 2, c->ruser))) return err;
        dt_cfl = -v[0];
      }
      dt = ORC_MIN(c->dt, dt_cfl);
    } else {
      dt = cfl_dt(c);
      if (c->reduce) {
        double v[2] = {-dt, -ORC_MAX_REAL};
        if ((err = c->reduce(v, 2, c->ruser))) return err;
        dt = -v[0];
      }
    }
    if (t + dt > t_next) dt = t_next - t;
    c->dt = dt;
    if ((err = advect_swarm(c))) return err;
    if (interpolated) {
      if ((err = partitions_setup(c))) return err;
      rbf_interpolation(c, c->cfg.nfields, c->fields);
    }
    if ((err = initialize_timestep_velocity(c))) return err;
    t += dt;
    c->nsteps++;
  }
  if (interpolated && !keep) {
    orc_reset_coefficients(c);
    /* CellInfoReset + clearing the data swarm (time_loop.c:94-98) */
    c->nd = 0;
    c->data_binned = 0;
  }
  return 0;
}

int orc_advect_interpolate(orc_ctx *c, double t, double t_next)
{
  if (!c->data_binned) return ORC_ERR_ARG_NULL;
  if (c->vfn || c->vfn_batch) return ORC_ERR_ARG_WRONGSTATE;
  return advection_loop(c, t, t_next, 1, 0);
}

int orc_advect_analytical(orc_ctx *c, double t, double t_next)
{
  if (!c->vfn && !c->vfn_batch) return ORC_ERR_ARG_NULL;
  return advection_loop(c, t, t_next, 0, 0);
}

int orc_set_velocity_fn(orc_ctx *c, orc_velocity_fn fn, void *user) { c->vfn = fn; c->vuser = user; return 0; }
int orc_set_velocity_batch_fn(orc_ctx *c, orc_velocity_batch_fn fn, void *user) { c->vfn_batch = fn; c->vuser = user; return 0; }
int orc_set_step_reduce(orc_ctx *c, orc_step_reduce_fn fn, void *user) { c->reduce = fn; c->ruser = user; return 0; }

int orc_get_counts(orc_ctx *c, int *nd, int *np_alive, int *npatch_setup, int *nsteps)
{
  int p, n = 0, s = 0;
  for (p = 0; p < c->np; p++) n += c->alive[p];
  for (p = 0; p < c->pu.nnodes; p++) s += c->patch_setup[p];
  if (nd) *nd = c->nd;
  if (np_alive) *np_alive = n;
  if (npatch_setup) *npatch_setup = s;
  if (nsteps) *nsteps = c->nsteps;
  return 0;
}

double orc_get_dt(orc_ctx *c) { return c->dt; }

int orc_get_cellids(orc_ctx *c, int is_data, int *cellid)
{
  int n = is_data ? c->nd : c->np;
  memcpy(cellid, is_data ? c->cell_d : c->cell_p, sizeof(int) * (size_t)n);
  return n;
}

long orc_get_patch_csr(orc_ctx *c, int *patch_start, int *patch_pts)
{
  return orc_patch_csr(&c->pu, c->cell_start, c->cell_pts, patch_start, patch_pts);
}

long orc_get_block_csr(orc_ctx *c, int *blk_start, int *blk_pts)
{
  return orc_block_csr(&c->pu, c->cell_start, c->cell_pts, blk_start, blk_pts);
}

int orc_get_weights(orc_ctx *c, double *weights)
{
  memcpy(weights, c->weights, sizeof(double) * (size_t)c->np * c->pu.nen);
  return c->np;
}

/* ======================================================================================= */
/* CPU baseline timing                                                                      */
/* ======================================================================================= */
static double now_s(void)
{
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

int orc_time_baseline(const orc_config *cfg, int nd, const double *xd, const double *fd, int np,
                      const double *xp, int nsteps, double dt, int nthreads, double *setup_s, double *step_s)
{
  int err = 0;
  double t0, t1, t2;
  int r;
  orc_ctx **ctxs;
  if (nthreads < 1) nthreads = 1;
  ctxs = (orc_ctx **)calloc((size_t)nthreads, sizeof(orc_ctx *));
  t0 = now_s();
  /* one emulated rank per thread: same dataset, disjoint particle subsets */
#pragma omp parallel for num_threads(nthreads) schedule(static, 1) reduction(| : err)
  for (r = 0; r < nthreads; r++) {
    int lo = (int)((long)np * r / nthreads), hi = (int)((long)np * (r + 1) / nthreads), e;
    orc_ctx *c = orc_create(cfg);
    ctxs[r] = c;
    if (!c) { err |= 1; continue; }
    e = orc_fill_swarm(c, 1, nd, xd, fd, NULL);
    if (!e) e = orc_fill_swarm(c, 0, hi - lo, &xp[(size_t)lo * cfg->dim], NULL, NULL);
    if (!e) e = orc_interpolation(c);
    err |= e;
  }
  t1 = now_s();
#pragma omp parallel for num_threads(nthreads) schedule(static, 1) reduction(| : err)
  for (r = 0; r < nthreads; r++) {
    orc_ctx *c = ctxs[r];
    int s, e = 0;
    double t = 0.0;
    if (!c) continue;
    /* steady state: the dataset, its binning and the patch factors stay resident (A_KSP) */
    for (s = 0; s < nsteps && !e; s++) {
      e = advection_loop(c, t, t + dt, 1, 1);
      t += dt;
    }
    err |= e;
  }
  t2 = now_s();
  for (r = 0; r < nthreads; r++) orc_destroy(ctxs[r]);
  free(ctxs);
  if (setup_s) *setup_s = t1 - t0;
  if (step_s) *step_s = t2 - t1;
  return err;
}

int orc_time_ranks(int nranks, const orc_config *cfgs, const int *nd, const double *const *xd,
                   const double *const *fd, const int *np, const double *const *xp, int nsteps, double dt,
                   double *setup_s, double *step_s, long *psteps)
{
  int err = 0, r;
  long ps = 0;
  double t0, t1, t2;
  orc_ctx **ctxs = (orc_ctx **)calloc((size_t)nranks, sizeof(orc_ctx *));
  t0 = now_s();
#pragma omp parallel for num_threads(nranks) schedule(static, 1) reduction(| : err)
  for (r = 0; r < nranks; r++) {
    orc_ctx *c = orc_create(&cfgs[r]);
    int e;
    ctxs[r] = c;
    if (!c) { err |= 1; continue; }
    e = orc_fill_swarm(c, 1, nd[r], xd[r], fd[r], NULL);
    if (!e) e = orc_fill_swarm(c, 0, np[r], xp[r], NULL, NULL);
    if (!e) e = orc_interpolation(c);
    err |= e;
  }
  t1 = now_s();
#pragma omp parallel for num_threads(nranks) schedule(static, 1) reduction(| : err) reduction(+ : ps)
  for (r = 0; r < nranks; r++) {
    orc_ctx *c = ctxs[r];
    int s, e = 0, p;
    double t = 0.0;
    if (!c) continue;
    for (s = 0; s < nsteps && !e; s++) {
      e = advection_loop(c, t, t + dt, 1, 1);
      t += dt;
      for (p = 0; p < c->np; p++) ps += c->alive[p];
    }
    err |= e;
  }
  t2 = now_s();
  for (r = 0; r < nranks; r++) orc_destroy(ctxs[r]);
  free(ctxs);
  if (setup_s) *setup_s = t1 - t0;
  if (step_s) *step_s = t2 - t1;
  if (psteps) *psteps = ps;
  return err;
}
