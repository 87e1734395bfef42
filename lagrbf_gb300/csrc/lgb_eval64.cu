/*
 * lgb_eval64.cu -- FP64 instantiations of the PU evaluation kernel (lgb_eval.cuh), the dispatcher
 * lgb_op_eval and the FP64 PU-weights kernel.
 */
#include "lgb_eval.cuh"
#include <string.h>
#include <stdlib.h>

extern "C" int lgb_eval32_launch_3d(const EvalParams *P, int fp, int ker, int stage, int grid, void *stream);
extern "C" int lgb_eval32_launch_2d(const EvalParams *P, int fp, int ker, int stage, int grid, void *stream);
extern "C" int lgb_build_records_3d(const EvalParams *P, int force, int grid, void *stream);
extern "C" int lgb_build_records_2d(const EvalParams *P, int force, int grid, void *stream);

/* Staging budgets (elements): FP32 gather 30 KB, FP32 record stream per stage from the measured
   table (lgb_eval_tune.h: stage count and size), FP64 48 KB. */
#define BUDGET32 7680
#include "lgb_eval_tune.h"
#define BUDGET32_TMA LGB_TMA_BUDGET_TUNED /* floats per staging round of the record kernel */
#define BUDGET64 6144
/* Polls of a bounded mbarrier wait of the evaluation kernel before it reports a timeout. */
#define EVAL_POLL_LIMIT (1 << 22)

template <int DIM, int FP>
static int launch64(const EvalParams &P, int grid, cudaStream_t s)
{
  static bool attr = false;
  size_t smem = (size_t)P.budget * sizeof(double);
  if (!attr) {
    cudaFuncSetAttribute(k_eval<double, DIM, FP, 1, KER_GENERIC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)smem);
    attr = true;
  }
  k_eval<double, DIM, FP, 1, KER_GENERIC><<<grid, P.chunk_cap, smem, s>>>(P);
  return (int)cudaGetLastError();
}

template <int DIM>
static int launch64_fp(const EvalParams &P, int fp, int grid, cudaStream_t s)
{
  switch (fp) {
  case 1: return launch64<DIM, 1>(P, grid, s);
  case 2: return launch64<DIM, 2>(P, grid, s);
  case 3: return launch64<DIM, 3>(P, grid, s);
  default: return launch64<DIM, 4>(P, grid, s);
  }
}

/* Floats per staging round: the measured table's value; LAGRBF_TMA_BUDGET overrides it for the
   tuner (lagrbf_gb300/tune_eval.py), which times every candidate without a rebuild. */
static int tma_budget(void)
{
  static int b = -1;
  if (b < 0) {
    const char *e = getenv("LAGRBF_TMA_BUDGET");
    b = (e && atoi(e) >= 256) ? (atoi(e) / 4) * 4 : BUDGET32_TMA;
  }
  return b;
}

/* Evaluate fields [nf_first, nf_first+nf) of the coefficient pool at every live particle and
   write them to out[p*out_stride + (f - nf_first)].  Fields are processed four at a time. */
extern "C" int lgb_op_eval(lgb_dev *d, int nf_first, int nf, double *out, int out_stride, void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  if (d->np <= 0 || nf <= 0) return 0;
  const lgb_geom &g = d->g;
  int grid = g.ncells + lgb_cdiv(d->np, d->chunk_cap) + 1;
  int ker = (g.kernel == LGB_KERNEL_WENDLAND_C2) ? KER_C2 : (g.kernel == LGB_KERNEL_GAUSSIAN) ? KER_GAUSS : KER_GENERIC;
  for (int f = nf_first; f < nf_first + nf; f += 4) {
    int fp = nf_first + nf - f;
    if (fp > 4) fp = 4;
    EvalParams P;
    P.g = g;
    P.cstart = d->cstart;
    P.xr32 = d->xr;
    P.xs64 = d->xs;
    P.c32 = d->c32;
    P.c64 = d->c64;
    P.coff = d->coff;
    P.slot = d->slot;
    P.setup = d->setup;
    P.F = d->F;
    P.f0 = f;
    P.pstart = d->pstart;
    P.plist = d->plist;
    P.chunk_start = d->chunk_start;
    P.xp = d->xp;
    P.out = out + (f - nf_first);
    P.out_stride = out_stride;
    P.ctrl = d->ctrl;
    P.chunk_cap = d->chunk_cap;
    P.rec32 = d->rec32;
    P.rec_off = d->rec_off;
    P.poll_limit = d->eval_poll_limit > 0 ? d->eval_poll_limit : EVAL_POLL_LIMIT;
    P.withhold_copies = d->eval_withhold;
    int rc;
    if (d->prec == LGB_PREC_FP32) {
      const int stage = (d->rec32 && f == 0 && fp == g.dim && d->rec_fp == g.dim) ? 1 : 0;
      P.budget = stage ? tma_budget() : BUDGET32;
      rc = (g.dim == 3) ? lgb_eval32_launch_3d(&P, fp, ker, stage, grid, stream)
                        : lgb_eval32_launch_2d(&P, fp, ker, stage, grid, stream);
    } else {
      P.budget = BUDGET64;
      rc = (g.dim == 3) ? launch64_fp<3>(P, fp, grid, s) : launch64_fp<2>(P, fp, grid, s);
    }
    lgb_count_launch(1);
    if (rc) return rc;
  }
  return 0;
}

/* (Re)build the precomputed FP32 record blocks; without `force` the kernel only runs when the
   preceding factorisation processed patches (device-side count). */
extern "C" int lgb_op_build_records(lgb_dev *d, int force, void *stream)
{
  if (!d->rec32 || d->F < d->g.dim) return 0;
  EvalParams P;
  memset(&P, 0, sizeof(P));
  P.g = d->g;
  P.cstart = d->cstart;
  P.xr32 = d->xr;
  P.xs64 = d->xs;
  P.c32 = d->c32;
  P.coff = d->coff;
  P.slot = d->slot;
  P.setup = d->setup;
  P.F = d->F;
  P.f0 = 0;
  P.ctrl = d->ctrl;
  P.rec32 = d->rec32;
  P.rec_off = d->rec_off;
  P.cdirty = d->cdirty;
  int grid = d->g.ncells < 8 * d->nsm ? d->g.ncells : 8 * d->nsm;
  int rc = (d->g.dim == 3) ? lgb_build_records_3d(&P, force, grid, stream) : lgb_build_records_2d(&P, force, grid, stream);
  lgb_count_launch(1);
  return rc;
}

extern "C" int lgb_op_weights(lgb_dev *d, double *w, void *stream)
{
  cudaStream_t s = (cudaStream_t)stream;
  if (d->np <= 0) return 0;
  if (d->g.dim == 3) k_weights<3><<<lgb_cdiv(d->np, 128), 128, 0, s>>>(d->g, d->np, d->xp, d->cell_p, d->alive, w);
  else k_weights<2><<<lgb_cdiv(d->np, 128), 128, 0, s>>>(d->g, d->np, d->xp, d->cell_p, d->alive, w);
  lgb_count_launch(1);
  return (int)cudaGetLastError();
}
