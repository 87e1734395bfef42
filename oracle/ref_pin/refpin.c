/*
 * refpin.c -- TEST INFRASTRUCTURE ONLY.  Array-backed stand-ins for the PETSc objects and the
 * LagRBF accessors that LagRBF's hot-loop translation units call, plus a flat C entry point per
 * unit, so the reference's own arithmetic can be run on the oracle's inputs:
 *
 *   rp_phi          KernelGetFunction / _AVX256 / _AVX512 (src/kernels/kernels_rbf.c:93-180)
 *   rp_weights      SwarmInterpSetWeights_AVX256 (src/swarm/weights_avx.c:97-243)
 *   rp_assemble     PartitionAssembleRBFMatrix_AVX512 (src/partitions/partition_asmb_avx512.c:119-198)
 *   rp_interpolate  PointwiseInterpolation_AVX512 / _AVX256 (src/interpolation/interpolation_avx512.c:121-291,
 *                   src/interpolation/interpolation_avx.c:104-266)
 *
 * Those units are compiled unmodified from the reference tree (see Makefile); this file defines
 * only what they call and does not restate their computations.  The objects hold what the units
 * read: the sequential DMDA's Q1 element -> node table and node coordinates (O + h*i, the uniform
 * coordinates of DMDASetUniformCoordinates), the swarm fields by name, dense matrices as plain
 * arrays, and per-patch / per-cell index lists supplied by the caller (the oracle's membership).
 */
#include <stdarg.h>

#include "petsc.h"
#include "lagrangian_rbf.h"
#include "partition_of_unity.h"
#include "partitions/partition.h"
#include "cell_info.h"
#include "kernels/kernels_rbf.h"

/* -------------------------------------------------------------------------------------------- */
/* PETSc stand-ins                                                                               */
/* -------------------------------------------------------------------------------------------- */
static char rp_msg[256];

PetscErrorCode rp_seterr(PetscErrorCode code, const char *fmt, ...)
{
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(rp_msg, sizeof(rp_msg), fmt, ap);
  va_end(ap);
  return code;
}

const char *rp_last_error(void) { return rp_msg; }

PetscErrorCode rp_calloc(size_t bytes, void **p)
{
  *p = calloc(bytes ? bytes : 1, 1);
  return *p ? 0 : 55;
}

PetscErrorCode PetscPrintf(MPI_Comm comm, const char *fmt, ...)
{
  (void)comm;
  (void)fmt;
  return 0;
}

struct rp_vec { PetscScalar *a; };
struct rp_mat { PetscScalar *a; };
struct rp_celldm { const char *coord_names[1]; const char *cellid_name; };

#define RP_MAX_FIELDS 4
struct rp_dm {
  /* DMDA part */
  PetscInt dim, nel, nen;
  const PetscInt *elements;
  struct rp_vec coords;
  /* DMSwarm part */
  PetscInt npoints;
  struct rp_celldm celldm;
  const char *fname[RP_MAX_FIELDS];
  void *fdata[RP_MAX_FIELDS];
  PetscInt fbs[RP_MAX_FIELDS];
  int nfield;
};

PetscErrorCode DMGetDimension(DM dm, PetscInt *dim) { *dim = dm->dim; return 0; }
PetscErrorCode DMGetCoordinateDM(DM dm, DM *cdm) { *cdm = dm; return 0; }
PetscErrorCode DMGetCoordinates(DM dm, Vec *c) { *c = &dm->coords; return 0; }
PetscErrorCode DMDAGetElements(DM dm, PetscInt *nel, PetscInt *nen, const PetscInt **e)
{
  *nel = dm->nel;
  *nen = dm->nen;
  *e = dm->elements;
  return 0;
}
PetscErrorCode DMDARestoreElements(DM dm, PetscInt *nel, PetscInt *nen, const PetscInt **e) { return 0; }
PetscErrorCode VecGetArray(Vec v, PetscScalar **a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArray(Vec v, PetscScalar **a) { return 0; }
PetscErrorCode MatDenseGetArray(Mat m, PetscScalar **a) { *a = m->a; return 0; }
PetscErrorCode MatDenseRestoreArray(Mat m, PetscScalar **a) { return 0; }
PetscErrorCode DMSwarmGetLocalSize(DM sw, PetscInt *n) { *n = sw->npoints; return 0; }
PetscErrorCode DMSwarmGetCellDMActive(DM sw, DMSwarmCellDM *c) { *c = &sw->celldm; return 0; }
PetscErrorCode DMSwarmCellDMGetCoordinateFields(DMSwarmCellDM c, PetscInt *nf, const char ***names)
{
  if (nf) *nf = 1;
  *names = c->coord_names;
  return 0;
}
PetscErrorCode DMSwarmCellDMGetCellID(DMSwarmCellDM c, const char **name) { *name = c->cellid_name; return 0; }
PetscErrorCode DMSwarmGetField(DM sw, const char *name, PetscInt *bs, PetscDataType *type, void **data)
{
  for (int i = 0; i < sw->nfield; i++)
    if (!strcmp(sw->fname[i], name)) {
      if (bs) *bs = sw->fbs[i];
      if (type) *type = 0;
      *data = sw->fdata[i];
      return 0;
    }
  return rp_seterr(PETSC_ERR_ARG_WRONG, "no swarm field %s", name);
}
PetscErrorCode DMSwarmRestoreField(DM sw, const char *name, PetscInt *bs, PetscDataType *type, void **data) { return 0; }

static void swarm_add(struct rp_dm *sw, const char *name, PetscInt bs, void *data)
{
  sw->fname[sw->nfield] = name;
  sw->fbs[sw->nfield] = bs;
  sw->fdata[sw->nfield] = data;
  sw->nfield++;
}

/* -------------------------------------------------------------------------------------------- */
/* LagRBF accessors called by the compiled units (plain field reads of the reference's structs)  */
/* -------------------------------------------------------------------------------------------- */
PetscErrorCode LagRBFGetPartitionOfUnity(LagRBFCtx ctx, PartitionOfUnity *pu) { *pu = ctx->pu; return 0; }
PetscErrorCode LagRBFGetPartitions(LagRBFCtx ctx, Partition **p) { *p = ctx->partitions; return 0; }
PetscErrorCode PUGetDMDALocal(PartitionOfUnity pu, DM *das) { *das = pu->das; return 0; }
PetscErrorCode PUGetDimension(PartitionOfUnity pu, PetscInt *dim) { *dim = pu->dim; return 0; }
PetscErrorCode PUGetNPartitionsLocal(PartitionOfUnity pu, PetscInt *npart) { *npart = pu->npart; return 0; }
PetscErrorCode PUGetGlobalToLocalElementMap(PartitionOfUnity pu, PetscInt **ptos) { *ptos = pu->ptos; return 0; }
PetscErrorCode PartitionGetDataPointsIdx(Partition p, PetscInt *ndata, PetscInt **idx)
{
  *ndata = p->ndata;
  *idx = p->data_idx;
  return 0;
}
PetscErrorCode PartitionGetCoefficientsMat(Partition p, Mat *X) { *X = p->X; return 0; }
PetscErrorCode PartitionGetRBFMatrix(Partition p, Mat *A) { *A = p->A; return 0; }
PetscErrorCode CellInfoGetDataPointsIdx(CellInfo ci, PetscInt *ndata, PetscInt **idx)
{
  *ndata = ci->ndata;
  *idx = ci->data_idx;
  return 0;
}

/* Units under test (declared here as the reference declares them in its headers/sources). */
PetscErrorCode SwarmInterpSetWeights_AVX256(LagRBFCtx ctx, DM sw);
PetscErrorCode PartitionAssembleRBFMatrix_AVX512(Partition p, PetscInt dim, PetscReal epsilon, PetscReal *coords,
                                                 KernelType ktype);
PetscErrorCode PointwiseInterpolation_AVX512(PartitionOfUnity pu, Partition *partitions, CellInfo *cellinfo,
                                             KernelType ktype, PetscInt nfields, PetscInt npoints_i, PetscInt *cellid_i,
                                             PetscReal *coords_i, PetscReal *coords_d, PetscReal *rbf_d,
                                             PetscReal *weights, PetscReal *values_i);
PetscErrorCode PointwiseInterpolation_AVX256(PartitionOfUnity pu, Partition *partitions, CellInfo *cellinfo,
                                          KernelType ktype, PetscInt nfields, PetscInt npoints_i, PetscInt *cellid_i,
                                          PetscReal *coords_i, PetscReal *coords_d, PetscReal *rbf_d,
                                          PetscReal *weights, PetscReal *values_i);

/* -------------------------------------------------------------------------------------------- */
/* mesh set-up: uniform DMDA with Q1 elements on one rank                                        */
/* -------------------------------------------------------------------------------------------- */
typedef struct {
  struct _p_PartitionOfUnity pu;
  struct rp_dm da;
  PetscInt n[3], *elements, *ptos;
  PetscReal O[3], L[3], *ncoords;
} rp_mesh;

static int mesh_init(rp_mesh *m, int dim, const int *n, const double *O, const double *L)
{
  memset(m, 0, sizeof(*m));
  int nn = 1, nc = 1;
  for (int d = 0; d < 3; d++) {
    m->n[d] = d < dim ? n[d] : 1;
    m->O[d] = d < dim ? O[d] : 0.0;
    m->L[d] = d < dim ? L[d] : 0.0;
    nn *= m->n[d];
    nc *= d < dim ? m->n[d] - 1 : 1;
  }
  int nen = 1 << dim;
  m->ncoords = malloc(sizeof(double) * (size_t)nn * dim);
  m->elements = malloc(sizeof(PetscInt) * (size_t)nc * nen);
  m->ptos = malloc(sizeof(PetscInt) * (size_t)nc);
  if (!m->ncoords || !m->elements || !m->ptos) return 55;
  /* nodes x-fastest; coordinate O + h*i with h = (L - O)/(n - 1) */
  for (int k = 0; k < m->n[2]; k++)
    for (int j = 0; j < m->n[1]; j++)
      for (int i = 0; i < m->n[0]; i++) {
        int id = i + m->n[0] * (j + m->n[1] * k), ijk[3] = {i, j, k};
        for (int d = 0; d < dim; d++)
          m->ncoords[(size_t)id * dim + d] = m->O[d] + (m->L[d] - m->O[d]) / (double)(m->n[d] - 1) * ijk[d];
      }
  /* Q1 elements x-fastest; corners (0,0),(1,0),(1,1),(0,1) on the lower face, then the upper face */
  static const int cx[4] = {0, 1, 1, 0}, cy[4] = {0, 0, 1, 1};
  int ncx = m->n[0] - 1, ncy = m->n[1] - 1, ncz = dim == 3 ? m->n[2] - 1 : 1;
  for (int k = 0; k < ncz; k++)
    for (int j = 0; j < ncy; j++)
      for (int i = 0; i < ncx; i++) {
        int e = i + ncx * (j + ncy * k);
        for (int c = 0; c < nen; c++) {
          int q = c & 3, z = c >> 2;
          m->elements[(size_t)e * nen + c] = (i + cx[q]) + m->n[0] * ((j + cy[q]) + m->n[1] * (k + z));
        }
        m->ptos[e] = e;
      }
  m->da.dim = dim;
  m->da.nel = nc;
  m->da.nen = nen;
  m->da.elements = m->elements;
  m->da.coords.a = m->ncoords;
  m->pu.das = &m->da;
  m->pu.dap = &m->da;
  m->pu.dim = dim;
  m->pu.n = m->n;
  m->pu.npart = nn;
  m->pu.npg = nn;
  m->pu.ptos = m->ptos;
  m->pu.O = m->O;
  m->pu.L = m->L;
  return 0;
}

static void mesh_free(rp_mesh *m)
{
  free(m->ncoords);
  free(m->elements);
  free(m->ptos);
}

/* -------------------------------------------------------------------------------------------- */
/* flat entry points                                                                             */
/* -------------------------------------------------------------------------------------------- */

/* phi(r_i) with the reference's scalar kernel (lanes == 1) or its AVX-256 / AVX-512 form
   (lanes == 4 / 8; n a multiple of lanes). */
int rp_phi(int kernel, int lanes, int n, const double *r, double eps, double *out)
{
  if (lanes == 1) {
    PetscReal (*fn)(PetscReal, PetscReal) = NULL;
    PetscCall(KernelGetFunction((KernelType)kernel, &fn));
    for (int i = 0; i < n; i++) out[i] = fn(r[i], eps);
    return 0;
  }
  if (lanes == 4) {
    __m256d (*fn)(__m256d, __m256d) = NULL;
    PetscCall(KernelGetFunction_AVX256((KernelType)kernel, &fn));
    for (int i = 0; i + 4 <= n; i += 4) _mm256_storeu_pd(out + i, fn(_mm256_loadu_pd(r + i), _mm256_set1_pd(eps)));
    return 0;
  }
  if (lanes == 8) {
    __m512d (*fn)(__m512d, __m512d) = NULL;
    PetscCall(KernelGetFunction_AVX512((KernelType)kernel, &fn));
    for (int i = 0; i + 8 <= n; i += 8) _mm512_storeu_pd(out + i, fn(_mm512_loadu_pd(r + i), _mm512_set1_pd(eps)));
    return 0;
  }
  return rp_seterr(PETSC_ERR_ARG_OUTOFRANGE, "lanes must be 1, 4 or 8");
}

/* Normalised corner weights weights[np*nen + k] of every point (all points inside the mesh). */
int rp_weights(int dim, const int *n, const double *O, const double *L, double eps_w, int np, const double *coords,
               const int *cellid, double *weights)
{
  rp_mesh m;
  int rc = mesh_init(&m, dim, n, O, L);
  if (rc) return rc;
  m.pu.epsilon_w = eps_w;
  int nn = m.pu.npart;
  struct _p_Partition *parts = calloc((size_t)nn, sizeof(*parts));
  Partition *pp = calloc((size_t)nn, sizeof(*pp));
  struct _p_LagRBFCtx ctx;
  struct rp_dm sw;
  memset(&ctx, 0, sizeof(ctx));
  memset(&sw, 0, sizeof(sw));
  if (!parts || !pp) { mesh_free(&m); free(parts); free(pp); return 55; }
  for (int i = 0; i < nn; i++) { parts[i].idx = i; pp[i] = &parts[i]; }
  ctx.pu = &m.pu;
  ctx.partitions = pp;
  sw.npoints = np;
  sw.celldm.coord_names[0] = "DMSwarmPIC_coor";
  sw.celldm.cellid_name = "DMSwarm_cellid";
  swarm_add(&sw, "DMSwarmPIC_coor", dim, (void *)coords);
  swarm_add(&sw, "DMSwarm_cellid", 1, (void *)cellid);
  swarm_add(&sw, "weights", 1 << dim, weights);
  rc = SwarmInterpSetWeights_AVX256(&ctx, &sw);
  free(parts);
  free(pp);
  mesh_free(&m);
  return rc;
}

/* Dense symmetric RBF matrix A[m*m] (row-major) of the points idx[0..m) of coords. */
int rp_assemble(int dim, int kernel, double eps, int m, const int *idx, const double *coords, double *A)
{
  struct _p_Partition p;
  struct rp_mat a = {A};
  memset(&p, 0, sizeof(p));
  p.A = &a;
  p.ndata = m;
  p.data_idx = (PetscInt *)idx;
  return PartitionAssembleRBFMatrix_AVX512(&p, dim, eps, (PetscReal *)coords, (KernelType)kernel);
}

/* Values at np points from the cell blocks (blk CSR), the patch lists (patch CSR) and column-major
   coefficients coeffs + coff[k] of every patch.  lanes 8: the AVX-512 loop, lanes 4: the AVX one. */
int rp_interpolate(int lanes, int dim, const int *n, const double *O, const double *L, double eps_r, int kernel,
                   int nd, const double *coords_d, const int *blk_start, const int *blk_pts, const int *patch_start,
                   const int *patch_pts, const double *coeffs, const long *coff, int nfields, int np,
                   const int *cellid, const double *coords_i, const double *weights, double *values)
{
  rp_mesh m;
  int rc = mesh_init(&m, dim, n, O, L);
  if (rc) return rc;
  m.pu.epsilon_r = eps_r;
  int nn = m.pu.npart, nc = m.da.nel;
  struct _p_Partition *parts = calloc((size_t)nn, sizeof(*parts));
  Partition *pp = calloc((size_t)nn, sizeof(*pp));
  struct rp_mat *mats = calloc((size_t)nn, sizeof(*mats));
  struct _p_CellInfo *cells = calloc((size_t)nc, sizeof(*cells));
  CellInfo *cp = calloc((size_t)nc, sizeof(*cp));
  double *rbf_d = calloc((size_t)(nd > 0 ? nd : 1), sizeof(double));
  if (!parts || !pp || !mats || !cells || !cp || !rbf_d) { rc = 55; goto done; }
  for (int i = 0; i < nn; i++) {
    parts[i].idx = i;
    parts[i].ndata = patch_start[i + 1] - patch_start[i];
    parts[i].data_idx = (PetscInt *)(patch_pts + patch_start[i]);
    mats[i].a = (PetscScalar *)(coeffs + coff[i]);
    parts[i].X = &mats[i];
    pp[i] = &parts[i];
  }
  for (int c = 0; c < nc; c++) {
    cells[c].idx = c;
    cells[c].ndata = blk_start[c + 1] - blk_start[c];
    cells[c].data_idx = (PetscInt *)(blk_pts + blk_start[c]);
    cp[c] = &cells[c];
  }
  if (lanes == 8)
    rc = PointwiseInterpolation_AVX512(&m.pu, pp, cp, (KernelType)kernel, nfields, np, (PetscInt *)cellid,
                                       (PetscReal *)coords_i, (PetscReal *)coords_d, rbf_d, (PetscReal *)weights, values);
  else if (lanes == 4)
    rc = PointwiseInterpolation_AVX256(&m.pu, pp, cp, (KernelType)kernel, nfields, np, (PetscInt *)cellid,
                                    (PetscReal *)coords_i, (PetscReal *)coords_d, rbf_d, (PetscReal *)weights, values);
  else
    rc = rp_seterr(PETSC_ERR_ARG_OUTOFRANGE, "lanes must be 4 or 8");
done:
  free(parts);
  free(pp);
  free(mats);
  free(cells);
  free(cp);
  free(rbf_d);
  mesh_free(&m);
  return rc;
}
