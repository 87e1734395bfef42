/*
 * lgb_bin.cu -- particle-to-cell binning, data-swarm arrangement and patch membership.
 *
 * Replaces, for one rank:
 *   DMSwarmPICSetCellId / DMLocatePoints (src/swarm/swarm_utils.c:995-1029) -> k_locate
 *   DMSwarmSortGetAccess / GetPointsPerCell                                -> counting sort
 *   PartitionCreate_PartitionToCellInverseMapping + PartitionFillDataPointsIdx
 *     (src/partitions/partition.c:54-87, 337-371)                          -> k_patch_sizes
 *   CellInfoCreateNeighbourElements + CellInfoFillDataIdx (src/cell_info.c:120-297, 468-501)
 *     -> the 3^dim neighbour walk of the evaluation kernel (no per-cell index copies)
 *
 * Membership is implicit: data points are stored in cell order (stable in fill index, the order
 * the oracle fixes for DMSwarmSortGetPointsPerCell), so patch k is the concatenation of the
 * contiguous ranges of its <= 2^dim adjacent cells in ascending cell index, and slot[k*8+s]
 * gives the offset of adjacent cell s inside the patch.
 */
#include "lgb_common.cuh"
#include <limits.h>

static long long g_launches = 0;
extern "C" void lgb_count_launch(long long n) { __atomic_add_fetch(&g_launches, n, __ATOMIC_RELAXED); }
extern "C" long long lgb_launch_count(void) { return __atomic_load_n(&g_launches, __ATOMIC_RELAXED); }

extern "C" int lgb_device_info(int *nsm, int *smem_optin)
{
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return (int)e;
  e = cudaDeviceGetAttribute(nsm, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return (int)e;
  e = cudaDeviceGetAttribute(smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  return (int)e;
}

/* ------------------------------------------------------------------------------------------- */
/* locate + histogram                                                                           */
/* ------------------------------------------------------------------------------------------- */
__global__ void k_locate(lgb_geom g, int n, const double *__restrict__ x, int *__restrict__ cell,
                         int *__restrict__ alive, int *__restrict__ counts, int *__restrict__ nbad,
                         const int *__restrict__ active)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (alive && !alive[i]) { cell[i] = -1; return; }
  int c = lgb_locate(g, x + (size_t)i * g.dim);
  cell[i] = c;
  if (c < 0) {
    if (alive) alive[i] = 0; /* DMSwarmMigrate on one rank drops points that left the domain */
    if (nbad) atomicAdd(nbad, 1);
    return;
  }
  if (counts && (!active || active[i])) atomicAdd(&counts[c], 1);
}

extern "C" int lgb_op_locate(const lgb_geom *g, int n, const double *x, int *cell, int *alive, int *counts,
                             int *nbad, void *stream)
{
  if (n <= 0) return 0;
  k_locate<<<lgb_cdiv(n, 256), 256, 0, (cudaStream_t)stream>>>(*g, n, x, cell, alive, counts, nbad, NULL);
  lgb_count_launch(1);
  LGB_CHECK_LAUNCH();
  return 0;
}

/* ------------------------------------------------------------------------------------------- */
/* exclusive scan: out[0..n], out[n] = total                                                     */
/* ------------------------------------------------------------------------------------------- */
#define SCAN_T 1024
#define SCAN_TILE (2 * SCAN_T)

template <typename T>
__device__ T block_exclusive_scan_pair(T a, T b, T *sh, T &total)
{
  /* each thread owns two consecutive elements (a, b); returns the exclusive prefix of a */
  int tid = threadIdx.x;
  T s = a + b;
  sh[tid] = s;
  __syncthreads();
  for (int off = 1; off < SCAN_T; off <<= 1) {
    T v = (tid >= off) ? sh[tid - off] : T(0);
    __syncthreads();
    sh[tid] += v;
    __syncthreads();
  }
  total = sh[SCAN_T - 1];
  T incl = sh[tid];
  __syncthreads();
  return incl - s;
}

template <typename T>
__global__ void k_scan_tiles(int n, const T *__restrict__ in, T *__restrict__ out, T *__restrict__ tile_sums)
{
  __shared__ T sh[SCAN_T];
  int base = blockIdx.x * SCAN_TILE + 2 * threadIdx.x;
  T a = (base < n) ? in[base] : T(0);
  T b = (base + 1 < n) ? in[base + 1] : T(0);
  T total;
  T ex = block_exclusive_scan_pair<T>(a, b, sh, total);
  if (base < n) out[base] = ex;
  if (base + 1 < n) out[base + 1] = ex + a;
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

template <typename T>
__global__ void k_scan_sums(int ntiles, T *__restrict__ tile_sums, T *__restrict__ out, int n)
{
  /* single CTA, ntiles <= SCAN_TILE */
  __shared__ T sh[SCAN_T];
  int base = 2 * threadIdx.x;
  T a = (base < ntiles) ? tile_sums[base] : T(0);
  T b = (base + 1 < ntiles) ? tile_sums[base + 1] : T(0);
  T total;
  T ex = block_exclusive_scan_pair<T>(a, b, sh, total);
  if (base < ntiles) tile_sums[base] = ex;
  if (base + 1 < ntiles) tile_sums[base + 1] = ex + a;
  if (threadIdx.x == 0) out[n] = total;
}

template <typename T>
__global__ void k_scan_add(int n, T *__restrict__ out, const T *__restrict__ tile_sums)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] += tile_sums[i / SCAN_TILE];
}

template <typename T>
static int scan_impl(int n, const T *in, T *out, T *tmp, cudaStream_t s)
{
  int ntiles = lgb_cdiv(n, SCAN_TILE);
  if (n <= 0) { cudaMemsetAsync(out, 0, sizeof(T), s); return (int)cudaGetLastError(); }
  if (ntiles > SCAN_TILE) return (int)cudaErrorInvalidValue; /* n <= 4M */
  k_scan_tiles<T><<<ntiles, SCAN_T, 0, s>>>(n, in, out, tmp);
  k_scan_sums<T><<<1, SCAN_T, 0, s>>>(ntiles, tmp, out, n);
  k_scan_add<T><<<lgb_cdiv(n, 256), 256, 0, s>>>(n, out, tmp);
  lgb_count_launch(3);
  LGB_CHECK_LAUNCH();
  return 0;
}

extern "C" int lgb_op_scan_i32(int n, const int *in, int *out, int *tmp, void *stream)
{
  return scan_impl<int>(n, in, out, tmp, (cudaStream_t)stream);
}
extern "C" int lgb_op_scan_i64(int n, const long long *in, long long *out, long long *tmp, void *stream)
{
  return scan_impl<long long>(n, in, out, tmp, (cudaStream_t)stream);
}

/* ------------------------------------------------------------------------------------------- */
/* scatter into per-cell lists                                                                  */
/* ------------------------------------------------------------------------------------------- */
__global__ void k_scatter(int n, const int *__restrict__ cell, const int *__restrict__ alive,
                          const int *__restrict__ start, int *__restrict__ fill, int *__restrict__ list,
                          const int *__restrict__ active)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (alive && !alive[i]) return;
  if (active && !active[i]) return;
  int c = cell[i];
  if (c < 0) return;
  int pos = start[c] + atomicAdd(&fill[c], 1);
  list[pos] = i;
}

extern "C" int lgb_op_scatter(int n, const int *cell, const int *alive, const int *start, int *fill, int *list,
                              void *stream)
{
  if (n <= 0) return 0;
  k_scatter<<<lgb_cdiv(n, 256), 256, 0, (cudaStream_t)stream>>>(n, cell, alive, start, fill, list, NULL);
  lgb_count_launch(1);
  LGB_CHECK_LAUNCH();
  return 0;
}

/* Sort each cell's segment ascending so that the data order inside a cell is the fill order
   (stable counting sort).  Segments up to SEG_SMEM entries are bitonic-sorted in shared memory;
   longer ones are ranked by counting. */
#define SEG_SMEM 4096
__global__ void k_segsort(int ncells, const int *__restrict__ start, int *__restrict__ list, int *__restrict__ tmp)
{
  __shared__ int sh[SEG_SMEM];
  int c = blockIdx.x;
  if (c >= ncells) return;
  int s0 = start[c], cnt = start[c + 1] - s0;
  if (cnt <= 1) return;
  if (cnt <= SEG_SMEM) {
    int p2 = 1;
    while (p2 < cnt) p2 <<= 1;
    for (int i = threadIdx.x; i < p2; i += blockDim.x) sh[i] = (i < cnt) ? list[s0 + i] : INT_MAX;
    __syncthreads();
    for (int k = 2; k <= p2; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int i = threadIdx.x; i < p2; i += blockDim.x) {
          int ixj = i ^ j;
          if (ixj > i) {
            bool up = ((i & k) == 0);
            int a = sh[i], b = sh[ixj];
            if ((a > b) == up) { sh[i] = b; sh[ixj] = a; }
          }
        }
        __syncthreads();
      }
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) list[s0 + i] = sh[i];
    return;
  }
  /* rank by counting (values are distinct point indices) */
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
    int v = list[s0 + i], r = 0;
    for (int q = 0; q < cnt; q++) r += (list[s0 + q] < v);
    tmp[s0 + r] = v;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < cnt; i += blockDim.x) list[s0 + i] = tmp[s0 + i];
}

/* ------------------------------------------------------------------------------------------- */
/* data swarm arrangement                                                                       */
/* ------------------------------------------------------------------------------------------- */
__global__ void k_gather_data(lgb_geom g, int nd, int F, const int *__restrict__ sorted, const int *__restrict__ cell,
                              const double *__restrict__ xd, const double *__restrict__ fd, double *__restrict__ xs,
                              float *__restrict__ xr, double *__restrict__ fs)
{
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nd) return;
  int i = sorted[s];
  int c = cell[i];
  int ci, cj, cl;
  lgb_cell_ijk(g, c, ci, cj, cl);
  int cc[3] = {ci, cj, cl};
  float r[4] = {0.f, 0.f, 0.f, 0.f};
  for (int d = 0; d < g.dim; d++) {
    double v = xd[(size_t)i * g.dim + d];
    if (xs) xs[(size_t)s * g.dim + d] = v;
    /* coordinate relative to the origin node of the point's own cell */
    r[d] = (float)(v - (g.O[d] + g.h[d] * cc[d]));
  }
  if (xr) reinterpret_cast<float4 *>(xr)[s] = make_float4(r[0], r[1], r[2], 0.f);
  if (fs)
    for (int f = 0; f < F; f++) fs[(size_t)s * F + f] = fd[(size_t)i * F + f];
}

/* Patch sizes and the offset of each adjacent cell inside the patch (ascending cell order). */
__global__ void k_patch_sizes(lgb_geom g, const int *__restrict__ cstart, int *__restrict__ pm,
                              int *__restrict__ slot, long long *__restrict__ pm64, int *__restrict__ maxm)
{
  int node = blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= g.nnodes) return;
  int nxy = g.n[0] * g.n[1];
  int l = node / nxy, r = node - l * nxy, j = r / g.n[0], i = r - j * g.n[0];
  int off = 0;
  int nslot = (g.dim == 3) ? 8 : 4;
  for (int s = 0; s < 8; s++) {
    int dx = s & 1, dy = (s >> 1) & 1, dz = (s >> 2) & 1;
    int ci = i - 1 + dx, cj = j - 1 + dy, cl = (g.dim == 3) ? (l - 1 + dz) : 0;
    slot[node * 8 + s] = off;
    if (s >= nslot) continue;
    if (ci < 0 || ci >= g.nc[0] || cj < 0 || cj >= g.nc[1] || cl < 0 || cl >= g.nc[2]) continue;
    int c = ci + cj * g.nc[0] + cl * g.nc[0] * g.nc[1];
    off += cstart[c + 1] - cstart[c];
  }
  pm[node] = off;
  pm64[node] = off;
  atomicMax(maxm, off);
}

__global__ void k_max_cell(int ncells, const int *__restrict__ cstart, int *__restrict__ out)
{
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  atomicMax(out, cstart[c + 1] - cstart[c]);
}

/* The data swarm: cell ids, stable cell order, arranged copies, patch sizes and offsets.
   d->xd, d->fd hold the filled arrays; the scratch pfill/scan buffers are reused. */
extern "C" int lgb_op_data_arrange(lgb_dev *d, void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  const lgb_geom &g = d->g;
  int nd = d->nd, rc;
  int *counts = d->pcount; /* ncells+1 scratch */
  cudaMemsetAsync(counts, 0, sizeof(int) * (g.ncells + 1), s);
  cudaMemsetAsync(d->dfill, 0, sizeof(int) * g.ncells, s);
  if ((rc = lgb_op_locate(&g, nd, d->xd, d->cell_d, NULL, counts, NULL, stream))) return rc;
  if ((rc = lgb_op_scan_i32(g.ncells, counts, d->cstart, d->scan_tmp, stream))) return rc;
  if ((rc = lgb_op_scatter(nd, d->cell_d, NULL, d->cstart, d->dfill, d->sorted, stream))) return rc;
  k_segsort<<<g.ncells, 256, 0, s>>>(g.ncells, d->cstart, d->sorted, d->dtmp);
  k_gather_data<<<lgb_cdiv(nd > 0 ? nd : 1, 256), 256, 0, s>>>(g, nd, d->F, d->sorted, d->cell_d, d->xd, d->fd,
                                                                d->xs, d->xr, d->fs);
  lgb_count_launch(2);
  LGB_CHECK_LAUNCH();
  /* patch sizes -> coefficient pool offsets */
  long long *pm64 = (long long *)d->need; /* borrowed: need[] holds 2*nnodes ints */
  int *maxm = &d->ctrl->nwork;             /* borrowed scalar; reset below */
  cudaMemsetAsync(maxm, 0, sizeof(int), s);
  k_patch_sizes<<<lgb_cdiv(g.nnodes, 128), 128, 0, s>>>(g, d->cstart, d->pm, d->slot, pm64, maxm);
  lgb_count_launch(1);
  LGB_CHECK_LAUNCH();
  if ((rc = lgb_op_scan_i64(g.nnodes, pm64, d->coff, d->scan_tmp64, stream))) return rc;
  cudaMemcpyAsync(&d->max_patch, maxm, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaMemsetAsync(maxm, 0, sizeof(int), s);
  k_max_cell<<<lgb_cdiv(g.ncells, 256), 256, 0, s>>>(g.ncells, d->cstart, maxm);
  cudaMemcpyAsync(&d->max_cell_pts, maxm, sizeof(int), cudaMemcpyDeviceToHost, s);
  cudaMemsetAsync(maxm, 0, sizeof(int), s);
  cudaMemsetAsync(d->need, 0, sizeof(int) * 2 * g.nnodes, s);
  lgb_count_launch(1);
  LGB_CHECK_LAUNCH();
  return (int)cudaStreamSynchronize(s);
}

/* Values changed, coordinates unchanged: refresh the cell-ordered copy only. */
__global__ void k_gather_values(int nd, int F, const int *__restrict__ sorted, const double *__restrict__ fd,
                                double *__restrict__ fs)
{
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nd) return;
  int i = sorted[s];
  for (int f = 0; f < F; f++) fs[(size_t)s * F + f] = fd[(size_t)i * F + f];
}

extern "C" int lgb_op_data_values(lgb_dev *d, void *stream)
{
  if (d->nd <= 0 || d->F <= 0) return 0;
  k_gather_values<<<lgb_cdiv(d->nd, 256), 256, 0, (cudaStream_t)stream>>>(d->nd, d->F, d->sorted, d->fd, d->fs);
  lgb_count_launch(1);
  LGB_CHECK_LAUNCH();
  return 0;
}

/* ------------------------------------------------------------------------------------------- */
/* particle binning per stage                                                                   */
/* ------------------------------------------------------------------------------------------- */
__global__ void k_chunks(int ncells, int cap, const int *__restrict__ pstart, int *__restrict__ nch)
{
  int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncells) return;
  nch[c] = lgb_cdiv(pstart[c + 1] - pstart[c], cap);
}

extern "C" int lgb_op_bin_particles(lgb_dev *d, int mark_dead, void *stream)
{
  return lgb_op_bin_particles_mask(d, mark_dead, NULL, stream);
}

extern "C" int lgb_op_bin_particles_mask(lgb_dev *d, int mark_dead, const int *active, void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  const lgb_geom &g = d->g;
  int rc;
  cudaMemsetAsync(d->pcount, 0, sizeof(int) * (g.ncells + 1), s);
  cudaMemsetAsync(d->pfill, 0, sizeof(int) * g.ncells, s);
  if (d->np > 0) {
    k_locate<<<lgb_cdiv(d->np, 256), 256, 0, s>>>(g, d->np, d->xp, d->cell_p, mark_dead ? d->alive : NULL, d->pcount,
                                                   NULL, active);
    lgb_count_launch(1);
    LGB_CHECK_LAUNCH();
  }
  if ((rc = lgb_op_scan_i32(g.ncells, d->pcount, d->pstart, d->scan_tmp, stream))) return rc;
  if (d->np > 0) {
    k_scatter<<<lgb_cdiv(d->np, 256), 256, 0, s>>>(d->np, d->cell_p, d->alive, d->pstart, d->pfill, d->plist, active);
    lgb_count_launch(1);
    LGB_CHECK_LAUNCH();
  }
  k_chunks<<<lgb_cdiv(g.ncells, 256), 256, 0, s>>>(g.ncells, d->chunk_cap, d->pstart, d->pfill);
  lgb_count_launch(1);
  LGB_CHECK_LAUNCH();
  return lgb_op_scan_i32(g.ncells, d->pfill, d->chunk_start, d->scan_tmp, stream);
}

/* ------------------------------------------------------------------------------------------- */
/* lazy patch set-up queue (LagRBF_PartitionsSetUp, partition.c:417-478)                        */
/* ------------------------------------------------------------------------------------------- */
__global__ void k_mark(lgb_geom g, int np, const int *__restrict__ cell, const int *__restrict__ alive,
                       const int *__restrict__ setup, const int *__restrict__ solved, int *__restrict__ need)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= np) return;
  if (!alive[p]) return;
  int c = cell[p];
  if (c < 0) return;
  int ci, cj, cl;
  lgb_cell_ijk(g, c, ci, cj, cl);
  for (int k = 0; k < g.nen; k++) {
    int ox, oy, oz;
    lgb_corner_offset(g.dim, k, ox, oy, oz);
    int node = (ci + ox) + (cj + oy) * g.n[0] + (cl + oz) * g.n[0] * g.n[1];
    if (!setup[node] || !solved[node]) need[node] = 1;
  }
}

/* Queued patches into the work-list region of their size class (cls_off); nwork counts them all.
   The cells around a queued patch node (up to 2^dim) are marked for a record rebuild. */
__global__ void k_compact(lgb_geom g, int *__restrict__ need, const int *__restrict__ pm,
                          const int *__restrict__ cls_off, int *__restrict__ work, lgb_ctrl *ctrl,
                          unsigned char *__restrict__ cdirty)
{
  int node = blockIdx.x * blockDim.x + threadIdx.x;
  if (node >= g.nnodes) return;
  if (need[node]) {
    need[node] = 0;
    const int c = lgb_patch_class(pm[node]);
    work[cls_off[c] + atomicAdd(&ctrl->nwork_c[c], 1)] = node;
    atomicAdd(&ctrl->nwork, 1);
    const int i = node % g.n[0], j = (node / g.n[0]) % g.n[1], k = node / (g.n[0] * g.n[1]);
    for (int dk = (g.dim == 3) ? -1 : 0; dk <= 0; dk++)
      for (int dj = -1; dj <= 0; dj++)
        for (int di = -1; di <= 0; di++) {
          const int a = i + di, b = j + dj, e = k + dk;
          if (a < 0 || b < 0 || e < 0 || a >= g.nc[0] || b >= g.nc[1] || e >= g.nc[2]) continue;
          cdirty[a + b * g.nc[0] + e * g.nc[0] * g.nc[1]] = 1;
        }
  }
}

/* Option setup_all_patches: every patch not yet set up or solved is queued. */
__global__ void k_mark_all(int nnodes, const int *__restrict__ setup, const int *__restrict__ solved,
                           int *__restrict__ need)
{
  int node = blockIdx.x * blockDim.x + threadIdx.x;
  if (node < nnodes && (!setup[node] || !solved[node])) need[node] = 1;
}

extern "C" int lgb_op_mark_patches(lgb_dev *d, void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(&d->ctrl->nwork, 0, sizeof(int), s);
  cudaMemsetAsync(d->ctrl->nwork_c, 0, sizeof(int) * LGB_NCLS, s);
  if (d->setup_all) {
    k_mark_all<<<lgb_cdiv(d->g.nnodes, 256), 256, 0, s>>>(d->g.nnodes, d->setup, d->solved, d->need);
    lgb_count_launch(1);
  } else if (d->np > 0) {
    k_mark<<<lgb_cdiv(d->np, 256), 256, 0, s>>>(d->g, d->np, d->cell_p, d->alive, d->setup, d->solved, d->need);
    lgb_count_launch(1);
  }
  k_compact<<<lgb_cdiv(d->g.nnodes, 256), 256, 0, s>>>(d->g, d->need, d->pm, d->cls_off_dev, d->work, d->ctrl,
                                                        d->cdirty);
  lgb_count_launch(1);
  LGB_CHECK_LAUNCH();
  return 0;
}

/* ------------------------------------------------------------------------------------------- */
/* output assembly by pid straight into the caller's host arrays                                */
/* ------------------------------------------------------------------------------------------- */
/* AssembleArray_Allreduce (src/interface/interface_utils.c:188-263) on one rank: row pid - 1 of
   each output holds the particle with that pid, rows of pids no longer in the swarm are zero.
   The rows are written by the GPU directly into host memory (devices that access pageable memory
   through the host's page tables, e.g. over NVLink-C2C), one pass, row-contiguous. */
__global__ void k_pid_inverse(int n, const long long *__restrict__ pid, const int *__restrict__ alive, int nglobal,
                              int *__restrict__ inv, int *__restrict__ bad)
{
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  if (alive && !alive[p]) return;
  long long gi = pid[p] - 1;
  if (gi < 0 || gi >= nglobal) {
    atomicExch(bad, 1);
    return;
  }
  inv[gi] = p;
}

/* Output rows gi of the caller's arrays (often pageable host memory reached through the GPU's
   address translation): a CTA gathers the rows of a tile of OUT_ROWS particles into shared memory,
   then writes each array's tile as one contiguous span, consecutive threads on consecutive words,
   so that every store fills whole sectors instead of a stride-dim pattern. */
#define OUT_ROWS 256
#define OUT_MAXW 8 /* words per row staged: dim <= 3, nf <= 8; wider rows are written directly */
__global__ void __launch_bounds__(OUT_ROWS) k_output_rows(int nglobal, const int *__restrict__ inv, int dim,
                                                          const double *__restrict__ x, double *coords, int nf,
                                                          const double *__restrict__ src, double *fields,
                                                          const long long *__restrict__ pid, long long *pidx)
{
  __shared__ double s_row[OUT_ROWS * OUT_MAXW];
  const int t = threadIdx.x;
  for (long long g0 = (long long)blockIdx.x * OUT_ROWS; g0 < nglobal; g0 += (long long)gridDim.x * OUT_ROWS) {
    const int nr = (int)min((long long)OUT_ROWS, (long long)nglobal - g0);
    const long long gi = g0 + t;
    const int p = (t < nr) ? inv[gi] : -1;
    if (pidx && t < nr) pidx[gi] = (p >= 0) ? pid[p] : 0;
    for (int a = 0; a < 2; a++) {
      const int w = a ? nf : dim;
      const double *in = a ? src : x;
      double *out = a ? fields : coords;
      if (!out || w <= 0) continue;
      if (w > OUT_MAXW) {
        if (t < nr)
          for (int k = 0; k < w; k++) out[gi * w + k] = (p >= 0) ? in[(size_t)p * w + k] : 0.0;
        continue;
      }
      if (t < nr)
        for (int k = 0; k < w; k++) s_row[t * w + k] = (p >= 0) ? in[(size_t)p * w + k] : 0.0;
      __syncthreads();
      double *o = out + g0 * w;
      for (int e = t; e < nr * w; e += OUT_ROWS) o[e] = s_row[e];
      __syncthreads();
    }
  }
}

extern "C" int lgb_op_output_rows(int n, const long long *pid, const int *alive, int nglobal, int *inv, int *bad,
                                  int dim, const double *x, double *coords, int nf, const double *src, double *fields,
                                  long long *pidx, int nsm, void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(inv, 0xff, sizeof(int) * (size_t)(nglobal > 0 ? nglobal : 1), s); /* -1: no particle */
  cudaMemsetAsync(bad, 0, sizeof(int), s);
  if (n > 0) k_pid_inverse<<<lgb_cdiv(n, 256), 256, 0, s>>>(n, pid, alive, nglobal, inv, bad);
  if (nglobal > 0) {
    int grid = lgb_cdiv(nglobal, OUT_ROWS);
    if (grid > 8 * nsm) grid = 8 * nsm;
    k_output_rows<<<grid, OUT_ROWS, 0, s>>>(nglobal, inv, dim, x, coords, nf, src, fields, pid, pidx);
  }
  lgb_count_launch(2);
  return (int)cudaGetLastError();
}

/* Host-to-device copy by the device itself, for host arrays it reads directly: 16-byte loads when
   both ends are 16-byte aligned, else 8-byte loads; consecutive threads on consecutive words. */
__global__ void k_copy_in(double *__restrict__ dst, const double *__restrict__ src, long long words, int vec)
{
  const long long stride = (long long)gridDim.x * blockDim.x;
  long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (vec) {
    const long long pairs = words / 2;
    const double2 *s2 = reinterpret_cast<const double2 *>(src);
    double2 *d2 = reinterpret_cast<double2 *>(dst);
    for (long long k = i; k < pairs; k += stride) d2[k] = s2[k];
    if (i == 0 && (words & 1)) dst[words - 1] = src[words - 1];
  } else {
    for (long long k = i; k < words; k += stride) dst[k] = src[k];
  }
}

/* DMSwarmAssignRankFromDMDA's bounding-box check (swarm_utils.c:854-871) of caller coordinates that
   the device reads directly, fused with the word-for-word comparison against the coordinates already
   on the device (prev, nullable): flags[0] = some point is outside [O, L], flags[1] = some word
   differs from prev.  One vote per warp, one atomic per warp that found something. */
__global__ void k_check_coords(lgb_geom g, int n, const double *x, const double *__restrict__ prev, int *flags)
{
  const int dim = g.dim;
  const long long stride = (long long)gridDim.x * blockDim.x;
  int out = 0, diff = 0;
  for (long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x; p < n; p += stride) {
    for (int d = 0; d < dim; d++) {
      const double v = x[p * dim + d];
      out |= (v < g.O[d]) | (v > g.L[d]); /* the host check's predicate (NaN passes, as there) */
      if (prev) diff |= __double_as_longlong(v) != __double_as_longlong(prev[p * dim + d]);
    }
  }
  const unsigned any_out = __ballot_sync(0xffffffffu, out), any_diff = __ballot_sync(0xffffffffu, diff);
  if ((threadIdx.x & 31) == 0) {
    if (any_out) atomicOr(&flags[0], 1);
    if (any_diff) atomicOr(&flags[1], 1);
  }
}

extern "C" int lgb_op_check_coords(const lgb_geom *g, int n, const double *x, const double *prev, int *flags, int nsm,
                                   void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  cudaMemsetAsync(flags, 0, 2 * sizeof(int), s);
  if (n > 0) {
    const long long need = ((long long)n + 255) / 256, cap = 8LL * (nsm > 0 ? nsm : 1);
    k_check_coords<<<(int)(need < cap ? need : cap), 256, 0, s>>>(*g, n, x, prev, flags);
    lgb_count_launch(1);
  }
  return (int)cudaGetLastError();
}

extern "C" int lgb_op_copy_in(double *dst, const double *src, long long words, int nsm, void *stream)
{
  if (words <= 0) return 0;
  const int vec = ((((uintptr_t)dst) | ((uintptr_t)src)) & 15) == 0;
  const long long items = vec ? words / 2 + 1 : words;
  const long long need = (items + 255) / 256, cap = 8LL * (nsm > 0 ? nsm : 1);
  const int grid = (int)(need < cap ? need : cap);
  k_copy_in<<<grid, 256, 0, (cudaStream_t)stream>>>(dst, src, words, vec);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}
