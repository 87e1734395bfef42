/*
 * lgb_eval_tune.h -- shared-memory staging of the FP32 record-streamed evaluation kernel,
 * measured by
 *     python -m lagrbf_gb300.tune_eval --np 16777216
 * (event-timed evaluation launches of the 3D RK4 workload: 128^3 jittered lattice, ABC flow,
 * 32^3 PU, Wendland C2, 16777216 uniform particles; ms per launch by stages x floats per stage):
 *   2 stages: 1024: 26.32, 1536: 25.37, 2048: 25.18, 2560: 25.34, 3072: 25.85
 *   3 stages: 1024: 26.42, 1536: 25.62, 2048: 26.43, 2560: 27.63, 3072: 29.97
 *   4 stages: 1024: 26.63, 1536: 27.03, 2048: 28.08, 2560: 30.63, 3072: 36.02
 */
#ifndef LGB_EVAL_TUNE_H
#define LGB_EVAL_TUNE_H
#define LGB_EVR_NB_TUNED 2
#define LGB_TMA_BUDGET_TUNED 2048
#endif
