/*
 * lgb_eval_tune.h -- shared-memory staging of the FP32 record-streamed evaluation kernel
 * (placeholder values until python -m lagrbf_gb300.tune_eval rewrites this file).
 */
#ifndef LGB_EVAL_TUNE_H
#define LGB_EVAL_TUNE_H
#define LGB_EVR_NB_TUNED 2
#define LGB_TMA_BUDGET_TUNED 2048
#endif
