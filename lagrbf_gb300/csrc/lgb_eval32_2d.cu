/*
 * lgb_eval32_2d.cu -- FP32-evaluation instantiations (2D) of the PU evaluation kernel (lgb_eval.cuh).
 */
#include "lgb_eval.cuh"

template <int DIM, int FP, int KER>
static int launch32(const EvalParams &P, int grid, cudaStream_t s)
{
  static bool attr = false;
  /* staging budget + per-thread running sums of the NEN*FP per-patch partial sums */
  size_t smem = ((size_t)P.budget + (size_t)(1 << DIM) * FP * LGB_CHUNK) * sizeof(float);
  if (!attr) {
    cudaFuncSetAttribute(k_eval<float, DIM, FP, 2, KER>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    attr = true;
  }
  k_eval<float, DIM, FP, 2, KER><<<grid, LGB_CHUNK / 2, smem, s>>>(P);
  return (int)cudaGetLastError();
}

template <int DIM, int KER>
static int launch32_fp(const EvalParams &P, int fp, int grid, cudaStream_t s)
{
  switch (fp) {
  case 1: return launch32<DIM, 1, KER>(P, grid, s);
  case 2: return launch32<DIM, 2, KER>(P, grid, s);
  case 3: return launch32<DIM, 3, KER>(P, grid, s);
  default: return launch32<DIM, 4, KER>(P, grid, s);
  }
}

extern "C" int lgb_eval32_launch_2d(const EvalParams *P, int fp, int ker, int grid, void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  if (ker == KER_C2) return launch32_fp<2, KER_C2>(*P, fp, grid, s);
  if (ker == KER_GAUSS) return launch32_fp<2, KER_GAUSS>(*P, fp, grid, s);
  return launch32_fp<2, KER_GENERIC>(*P, fp, grid, s);
}
