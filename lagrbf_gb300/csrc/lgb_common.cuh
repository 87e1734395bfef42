/*
 * lgb_common.cuh -- device helpers shared by the CUDA translation units.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>
#include "lgb_internal.h"

#define LGB_CHECK_LAUNCH() do { cudaError_t e__ = cudaGetLastError(); if (e__ != cudaSuccess) return (int)e__; } while (0)

/* Counts every kernel launch of the library (the benchmark reports it as gpu_launches). */
extern "C" void lgb_count_launch(long long n);

__host__ __device__ static inline int lgb_cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

/* Order-preserving integer key of a double: a < b  <=>  key(a) < key(b) for non-NaN values, with
   -0 and +0 equal; NaNs land beyond +inf or below -inf, i.e. outside any [O, L]. */
__host__ __device__ __forceinline__ long long lgb_key(double v)
{
  long long b;
  memcpy(&b, &v, sizeof b);
  if (b == (long long)0x8000000000000000ULL) b = 0;
  return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}

/* Cell of a point on the uniform PU mesh (DMSwarmPICSetCellId / DMLocatePoints on a uniform DMDA,
   the convention the oracle fixes): -1 outside [O, L] or NaN, else per axis
   clamp(floor((x - O) / h), 0, n - 2) in FP64, x == L in the last cell.  With the face keys the same index is the number
   of faces at or below x (integer binary search; the FP64 division and floor would keep GB300's
   FP64 pipe, 1/64 of the FP32 rate, busy for the whole launch). */
__device__ __forceinline__ int lgb_locate(const lgb_geom &g, const double *x)
{
  int c[3] = {0, 0, 0};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (d >= g.dim) break;
    double xd = x[d];
    if (g.bkey) {
      const long long k = lgb_key(xd);
      if (k < g.okey[d] || k > g.lkey[d]) return -1;
      const long long *b = g.bkey + g.boff[d];
      int lo = 0, hi = g.n[d] - 2; /* faces b[0 .. n-3]; the answer is how many are <= k */
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(b + mid) <= k) lo = mid + 1; else hi = mid;
      }
      c[d] = lo;
    } else {
      if (!(xd >= g.O[d] && xd <= g.L[d])) return -1;
      int t = (int)floor((xd - g.O[d]) / g.h[d]);
      if (t > g.n[d] - 2) t = g.n[d] - 2;
      if (t < 0) t = 0;
      c[d] = t;
    }
  }
  return c[0] + c[1] * g.nc[0] + c[2] * g.nc[0] * g.nc[1];
}

__device__ __forceinline__ void lgb_cell_ijk(const lgb_geom &g, int cell, int &i, int &j, int &l)
{
  int cxy = g.nc[0] * g.nc[1];
  l = cell / cxy;
  int r = cell - l * cxy;
  j = r / g.nc[0];
  i = r - j * g.nc[0];
}

/* Q1 corner k of a cell in PETSc's DMDAGetElements order (lower face counter-clockwise, then the
   upper face).  Returns the (x, y, z) node offsets. */
__host__ __device__ __forceinline__ void lgb_corner_offset(int dim, int k, int &ox, int &oy, int &oz)
{
  /* 0:(0,0,0) 1:(1,0,0) 2:(1,1,0) 3:(0,1,0) 4..7 same with z+1 */
  int q = k & 3;
  ox = (q == 1 || q == 2) ? 1 : 0;
  oy = (q >= 2) ? 1 : 0;
  oz = (dim == 3) ? (k >> 2) : 0;
}

/* RBF kernels of kernels_rbf.c:31-91, in the operation order of the reference's vector forms. */
template <typename T>
__device__ __forceinline__ T lgb_phi(int kernel, T r, T eps)
{
  T u, u2;
  switch (kernel) {
  case LGB_KERNEL_LINEAR: return eps * r;
  case LGB_KERNEL_WENDLAND_C0: u = T(1) - eps * r; u = (u >= T(0)) ? u : T(0); return u * u;
  case LGB_KERNEL_WENDLAND_C2:
    u = T(1) - eps * r;
    if (!(u >= T(0))) return T(0);
    u2 = u * u;
    return (u2 * u2) * (T(5) - T(4) * u);
  case LGB_KERNEL_BUMP:
    u = T(1) - eps * r;
    if (!(u >= T(0))) return T(0);
    return exp(T(-1) / (u * (T(2) - u)));
  case LGB_KERNEL_MQ: u = eps * r; return sqrt(T(1) + u * u);
  case LGB_KERNEL_IMQ: u = eps * r; return T(1) / sqrt(T(1) + u * u);
  case LGB_KERNEL_GAUSSIAN: u = eps * r; return exp(-(u * u));
  default: return T(0);
  }
}

/* Wendland C2 without the kernel switch (PU weights, swarm_interp.c:349). */
template <typename T>
__device__ __forceinline__ T lgb_wendland_c2(T r, T eps)
{
  T u = T(1) - eps * r;
  if (!(u >= T(0))) return T(0);
  T u2 = u * u;
  return (u2 * u2) * (T(5) - T(4) * u);
}

/* Error-free transformation of a sum (Knuth's TwoSum). */
__device__ __forceinline__ void lgb_two_sum(float a, float b, float &s, float &e)
{
  s = a + b;
  float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}

/* Double-float accumulate: (hi, lo) += x. */
__device__ __forceinline__ void lgb_df_add(float &hi, float &lo, float x)
{
  float s, e;
  lgb_two_sum(hi, x, s, e);
  lo += e;
  hi = s;
}
