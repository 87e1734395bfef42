/*
 * lgb_noalloc.cu -- binning of points into the cells of the PU mesh without any device allocation.
 *
 * Some callers cannot let a library allocate device memory at the point where they bin: a host
 * simulation code that reserves all of its device memory at start-up and runs its time loop from
 * a fixed pool (a cudaMalloc there would exceed the reservation and, being synchronising, stall its
 * other streams), or a caller that records its time step into its own stream capture, where a
 * cudaMalloc of ours is not allowed.  For them this file offers the particle/data binning of the
 * context path (locate, per-cell counts, exclusive scan, scatter, stable per-cell order) with all
 * of its scratch in one statically sized device array of this module instead of buffers owned by a
 * context.  The caller passes device buffers for the results; nothing here calls cudaMalloc,
 * cudaFree or any allocating library.
 *
 * Scratch: per-cell counters / cursors for at most LAGRBF_NOALLOC_MAX_CELLS cells (4 MiB) plus one
 * block total per 1024 cells.  The counters must start at zero: every call clears the first ncells
 * of them on the stream before counting, so nothing is carried over from an earlier call.
 *
 * The scratch array is shared by every call on a device.  Calls whose work overlaps on the device
 * (different streams, or several host threads without ordering) race on it and give wrong
 * results; issue them on one stream, or order them with events.
 *
 * Set-up: the first call on a device (with that device current) resolves the scratch array's
 * address with cudaGetSymbolAddress, which may load this module; that call should therefore come
 * before any stream capture the caller begins.
 */
#include <mutex>
#include <stdio.h>
#include <string.h>

#include "lgb_common.cuh"
#include "../../include/lagrbf.h"

#define NA_MAX_CELLS LAGRBF_NOALLOC_MAX_CELLS
#define NA_SCAN_BLOCK 1024
#define NA_NBLK (NA_MAX_CELLS / NA_SCAN_BLOCK)
#define NA_SEG_SMEM 4096
#define NA_MAX_DEVICES 64

static_assert(NA_MAX_CELLS % NA_SCAN_BLOCK == 0, "scan blocks tile the cell range");
static_assert(NA_NBLK <= NA_SCAN_BLOCK, "block totals are scanned by one block");

/* [0, NA_MAX_CELLS): per-cell counters, then cursors; [NA_MAX_CELLS, +NA_NBLK): scan block totals. */
static __device__ __align__(256) int g_na_scratch[NA_MAX_CELLS + NA_NBLK];

static int *g_na_ptr[NA_MAX_DEVICES];
static std::mutex g_na_lock;

__global__ void k_na_zero(int n, int *__restrict__ cnt)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) cnt[i] = 0;
}

__global__ void k_na_count(lgb_geom g, int np, const double *__restrict__ x, int *__restrict__ cellid,
                           int *__restrict__ cnt)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  int c = lgb_locate(g, x + (size_t)i * g.dim);
  cellid[i] = c;
  if (c >= 0) atomicAdd(&cnt[c], 1);
}

/* Exclusive scan of 1024 counters per block; block totals to bsum. */
__global__ void k_na_scan_block(int n, const int *__restrict__ cnt, int *__restrict__ start, int *__restrict__ bsum)
{
  __shared__ int warp_tot[32];
  int i = blockIdx.x * NA_SCAN_BLOCK + threadIdx.x;
  int v = (i < n) ? cnt[i] : 0;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int s = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += t;
  }
  if (lane == 31) warp_tot[w] = s;
  __syncthreads();
  if (w == 0) {
    int t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int u = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += u;
    }
    warp_tot[lane] = t; /* inclusive over warps */
  }
  __syncthreads();
  int excl = s - v + (w > 0 ? warp_tot[w - 1] : 0);
  if (i < n) start[i] = excl;
  if (threadIdx.x == NA_SCAN_BLOCK - 1) bsum[blockIdx.x] = warp_tot[31];
}

/* Exclusive scan of the block totals in place (one block); the grand total to start[n]. */
__global__ void k_na_scan_top(int nblk, int n, int *__restrict__ bsum, int *__restrict__ start)
{
  __shared__ int warp_tot[32];
  int v = ((int)threadIdx.x < nblk) ? bsum[threadIdx.x] : 0;
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int s = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    int t = __shfl_up_sync(0xffffffffu, s, o);
    if (lane >= o) s += t;
  }
  if (lane == 31) warp_tot[w] = s;
  __syncthreads();
  if (w == 0) {
    int t = warp_tot[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int u = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += u;
    }
    warp_tot[lane] = t;
  }
  __syncthreads();
  int excl = s - v + (w > 0 ? warp_tot[w - 1] : 0);
  if ((int)threadIdx.x < nblk) bsum[threadIdx.x] = excl;
  if (threadIdx.x == 0) start[n] = warp_tot[31];
}

/* Adds the block offsets; the counters become the scatter cursors. */
__global__ void k_na_scan_add(int n, int *__restrict__ start, const int *__restrict__ bsum, int *__restrict__ cur)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  int s = start[i] + bsum[i / NA_SCAN_BLOCK];
  start[i] = s;
  cur[i] = s;
}

__global__ void k_na_scatter(int np, const int *__restrict__ cellid, int *__restrict__ cur, int *__restrict__ order)
{
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  int c = cellid[i];
  if (c >= 0) order[atomicAdd(&cur[c], 1)] = i;
}

/* Ascending sort of v[0, cnt) by one block: bitonic network in its all-ascending form (the first
   step of every merge compares mirrored positions), so positions >= cnt act as +infinity that
   never move and are skipped. */
__device__ void na_sort_ascending(int *v, int cnt)
{
  int p2 = 1;
  while (p2 < cnt) p2 <<= 1;
  int npair = p2 >> 1;
  for (int k = 2; k <= p2; k <<= 1) {
    int half = k >> 1;
    for (int t = threadIdx.x; t < npair; t += blockDim.x) {
      int blk = t / half, off = t - blk * half;
      int a = blk * k + off, b = blk * k + k - 1 - off;
      if (b < cnt) {
        int va = v[a], vb = v[b];
        if (va > vb) { v[a] = vb; v[b] = va; }
      }
    }
    __syncthreads();
    for (int j = k >> 2; j > 0; j >>= 1) {
      for (int t = threadIdx.x; t < npair; t += blockDim.x) {
        int blk = t / j, off = t - blk * j;
        int a = blk * 2 * j + off, b = a + j;
        if (b < cnt) {
          int va = v[a], vb = v[b];
          if (va > vb) { v[a] = vb; v[b] = va; }
        }
      }
      __syncthreads();
    }
  }
}

/* One block per cell: the cell's point indices in ascending (= input) order. */
__global__ void k_na_segsort(int ncells, const int *__restrict__ start, int *__restrict__ order)
{
  __shared__ int sh[NA_SEG_SMEM];
  int c = blockIdx.x;
  int s0 = start[c], cnt = start[c + 1] - s0;
  if (cnt <= 1) return;
  if (cnt <= NA_SEG_SMEM) {
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) sh[i] = order[s0 + i];
    __syncthreads();
    na_sort_ascending(sh, cnt);
    for (int i = threadIdx.x; i < cnt; i += blockDim.x) order[s0 + i] = sh[i];
    return;
  }
  na_sort_ascending(order + s0, cnt);
}

static int na_fail(int code, const char *what, cudaError_t e)
{
  char msg[256];
  snprintf(msg, sizeof(msg), "lagrbf_gpu_bin_points_noalloc: %s%s%s", what, e != cudaSuccess ? ": " : "",
           e != cudaSuccess ? cudaGetErrorString(e) : "");
  return lgb_set_error_msg(code, msg);
}

/* Scratch address on the current device, resolved once per device and kept for the life of the
   process: after cudaDeviceReset, or in a context other than the device's primary context, the
   kept address is stale and the entry point must not be used. */
static int na_scratch(int **ptr)
{
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return na_fail(LAGRBF_ERR_GPU, "cudaGetDevice failed", e);
  if (dev < 0 || dev >= NA_MAX_DEVICES) return na_fail(LAGRBF_ERR_SUP, "device ordinal beyond the set-up table", cudaSuccess);
  std::lock_guard<std::mutex> lock(g_na_lock);
  if (!g_na_ptr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_na_scratch);
    if (e != cudaSuccess || !p) return na_fail(LAGRBF_ERR_GPU, "cudaGetSymbolAddress of the scratch array failed", e);
    g_na_ptr[dev] = (int *)p;
  }
  *ptr = g_na_ptr[dev];
  return 0;
}

extern "C" LAGRBF_EXPORT int lagrbf_gpu_bin_points_noalloc(int32_t dim, const int32_t *nodes, const double *O,
                                                           const double *L, int32_t npoints, const double *coords,
                                                           int32_t *cellid, int32_t *cell_start, int32_t *order,
                                                           void *stream)
{
  if (dim != 2 && dim != 3) return na_fail(LAGRBF_ERR_ARG_OUTOFRANGE, "dim must be 2 or 3", cudaSuccess);
  if (!nodes || !O || !L || !cell_start) return na_fail(LAGRBF_ERR_ARG_NULL, "NULL geometry or cell_start", cudaSuccess);
  if (npoints < 0) return na_fail(LAGRBF_ERR_ARG_SIZ, "negative npoints", cudaSuccess);
  if (npoints > 0 && (!coords || !cellid || !order))
    return na_fail(LAGRBF_ERR_ARG_NULL, "NULL coords, cellid or order", cudaSuccess);
  lgb_geom g;
  memset(&g, 0, sizeof(g));
  g.dim = dim;
  g.nen = 1 << dim;
  long long ncells = 1;
  for (int i = 0; i < 3; i++) {
    if (i < dim) {
      if (nodes[i] < 2) return na_fail(LAGRBF_ERR_ARG_OUTOFRANGE, "nodes per axis must be >= 2", cudaSuccess);
      if (!(L[i] > O[i])) return na_fail(LAGRBF_ERR_ARG_OUTOFRANGE, "L must exceed O on every axis", cudaSuccess);
      g.n[i] = nodes[i];
      g.nc[i] = nodes[i] - 1;
      g.O[i] = O[i];
      g.L[i] = L[i];
      g.h[i] = (L[i] - O[i]) / (double)(nodes[i] - 1);
      ncells *= nodes[i] - 1;
    } else {
      g.n[i] = 1; g.nc[i] = 1; g.O[i] = 0; g.L[i] = 0; g.h[i] = 1.0;
    }
    if (ncells > NA_MAX_CELLS) break;
  }
  if (ncells > NA_MAX_CELLS) {
    char msg[160];
    snprintf(msg, sizeof(msg), "the mesh has more than %d cells, the size of the static scratch", NA_MAX_CELLS);
    return na_fail(LAGRBF_ERR_ARG_OUTOFRANGE, msg, cudaSuccess);
  }
  g.ncells = (int)ncells;
  g.nnodes = g.n[0] * g.n[1] * g.n[2];

  int *scratch = nullptr;
  int rc = na_scratch(&scratch);
  if (rc) return rc;
  int *cnt = scratch, *bsum = scratch + NA_MAX_CELLS;
  cudaStream_t s = (cudaStream_t)stream;
  int nc = g.ncells, nblk = lgb_cdiv(nc, NA_SCAN_BLOCK);

  k_na_zero<<<lgb_cdiv(nc, 256) < 1024 ? lgb_cdiv(nc, 256) : 1024, 256, 0, s>>>(nc, cnt);
  if (npoints > 0) k_na_count<<<lgb_cdiv(npoints, 256), 256, 0, s>>>(g, npoints, coords, cellid, cnt);
  k_na_scan_block<<<nblk, NA_SCAN_BLOCK, 0, s>>>(nc, cnt, cell_start, bsum);
  k_na_scan_top<<<1, NA_SCAN_BLOCK, 0, s>>>(nblk, nc, bsum, cell_start);
  k_na_scan_add<<<lgb_cdiv(nc, 256), 256, 0, s>>>(nc, cell_start, bsum, cnt);
  if (npoints > 0) {
    k_na_scatter<<<lgb_cdiv(npoints, 256), 256, 0, s>>>(npoints, cellid, cnt, order);
    k_na_segsort<<<nc, 256, 0, s>>>(nc, cell_start, order);
  }
  lgb_count_launch(npoints > 0 ? 7 : 4);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return na_fail(LAGRBF_ERR_GPU, "kernel launch failed", e);
  return 0;
}
