/*
 * lgb_eval32_2d.cu -- FP32-evaluation instantiations of the PU evaluation kernel (lgb_eval.cuh), 2D.
 */
#include "lgb_evalrec.cuh"
#include <stdlib.h>

template <int DIM, int FP, int KER, int R>
static int launch32r(const EvalParams &P, int grid, cudaStream_t s)
{
  static bool attr = false;
  const int nbuf = 1;
  /* staging buffer(s) + per-thread running sums of the R*NEN*FP per-patch partial sums */
  size_t smem = ((size_t)nbuf * P.budget + (size_t)(R * (1 << DIM) * FP + 1) * (P.chunk_cap / R)) * sizeof(float);
  if (!attr) {
    size_t smax = ((size_t)nbuf * P.budget + (size_t)(R * (1 << DIM) * FP + 1) * (LGB_CHUNK_MAX / R)) * sizeof(float);
    cudaFuncSetAttribute(k_eval<float, DIM, FP, R, KER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smax);
    attr = true;
  }
  k_eval<float, DIM, FP, R, KER><<<grid, P.chunk_cap / R, smem, s>>>(P);
  return (int)cudaGetLastError();
}

/* Two particles per thread (four per thread measured slower: fewer active lanes per work unit). */
template <int DIM, int FP, int KER>
static int launch32(const EvalParams &P, int grid, cudaStream_t s)
{
  return launch32r<DIM, FP, KER, 2>(P, grid, s);
}

/* The record-streamed kernel: EVR_NB stages of P.budget floats, then the PU-weight pairs. */
template <int DIM, int KER>
static int launch_rec(const EvalParams &P, int grid, cudaStream_t s)
{
  /* the attribute is set once to the device's largest opt-in size (threads racing on it all set the
     same value; a per-call size could shrink it under another thread's launch) */
  static int attr = 0;
  const size_t smem = (size_t)EVR_NB * P.budget * sizeof(float) + (size_t)(P.chunk_cap / 2) * ((1 << DIM) + 1) * 8;
  if (!attr) {
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    cudaFuncSetAttribute(k_eval_rec<DIM, DIM, KER>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         optin - 8192);
    attr = 1;
  }
  k_eval_rec<DIM, DIM, KER><<<grid, P.chunk_cap / 2, smem, s>>>(P);
  return (int)cudaGetLastError();
}

template <int DIM, int KER>
static int launch32_fp(const EvalParams &P, int fp, int stage, int grid, cudaStream_t s)
{
  if (stage == 1) return launch_rec<DIM, KER>(P, grid, s); /* records hold the dim velocity fields */
  switch (fp) {
  case 1: return launch32<DIM, 1, KER>(P, grid, s);
  case 2: return launch32<DIM, 2, KER>(P, grid, s);
  case 3: return launch32<DIM, 3, KER>(P, grid, s);
  default: return launch32<DIM, 4, KER>(P, grid, s);
  }
}

extern "C" int lgb_eval32_launch_2d(const EvalParams *P, int fp, int ker, int stage, int grid, void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  if (ker == KER_C2) return launch32_fp<2, KER_C2>(*P, fp, stage, grid, s);
  if (ker == KER_GAUSS) return launch32_fp<2, KER_GAUSS>(*P, fp, stage, grid, s);
  return launch32_fp<2, KER_GENERIC>(*P, fp, stage, grid, s);
}

extern "C" int lgb_build_records_2d(const EvalParams *P, int force, int grid, void *stream)
{
  k_build_records2<2, 2><<<grid, 128, 0, (cudaStream_t)stream>>>(*P, force);
  return (int)cudaGetLastError();
}
