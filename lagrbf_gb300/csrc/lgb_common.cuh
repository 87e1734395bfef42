/*
 * lgb_common.cuh -- device helpers shared by the CUDA translation units.
 */
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "lgb_internal.h"

#define LGB_CHECK_LAUNCH() do { cudaError_t e__ = cudaGetLastError(); if (e__ != cudaSuccess) return (int)e__; } while (0)

/* Counts every kernel launch of the library (the benchmark reports it as gpu_launches). */
extern "C" void lgb_count_launch(long long n);

__host__ __device__ static inline int lgb_cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

/* Cell of a point on the uniform PU mesh; -1 when outside [O, L] (or NaN).  Per axis
   floor((x - O)/h) in FP64, x == L mapped to the last cell -- the convention the oracle fixes for
   PETSc's DMLocatePoints on a uniform DMDA. */
__device__ __forceinline__ int lgb_locate(const lgb_geom &g, const double *x)
{
  int c[3] = {0, 0, 0};
#pragma unroll
  for (int d = 0; d < 3; d++) {
    if (d >= g.dim) break;
    double xd = x[d];
    if (!(xd >= g.O[d] && xd <= g.L[d])) return -1;
    int t = (int)floor((xd - g.O[d]) / g.h[d]);
    if (t > g.n[d] - 2) t = g.n[d] - 2;
    if (t < 0) t = 0;
    c[d] = t;
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
