/*
 * lgb_factor_tune.h -- CTA size of the patch set-up / solve launch of each patch-size class
 * (classes of up to 32, 64, 128, 256, 512, 1024, 2048 points and beyond), measured by
 *     python -m lagrbf_gb300.tune_factor
 * (event-timed set-up of every patch of a synthetic dataset per class, CTA sizes 32-256):
 *   class 0 (<= 32): 32: 0.7 ms, 64: 0.7 ms, 128: 0.8 ms, 256: 1.0 ms -> 32
 *   class 1 (<= 64): 32: 1.3 ms, 64: 1.4 ms, 128: 1.5 ms, 256: 1.7 ms -> 32
 *   class 2 (<= 128): 32: 4.1 ms, 64: 4.0 ms, 128: 4.0 ms, 256: 4.0 ms -> 64
 *   class 3 (<= 256): 32: 15.3 ms, 64: 15.0 ms, 128: 15.8 ms, 256: 14.2 ms -> 256
 *   class 4 (<= 512): 32: 60.0 ms, 64: 33.4 ms, 128: 21.9 ms, 256: 21.3 ms -> 256
 *   class 5 (<= 1024): 32: 289.6 ms, 64: 163.7 ms, 128: 115.2 ms, 256: 109.0 ms -> 256
 *   class 6 (<= 2048): 32: 1873.0 ms, 64: 957.8 ms, 128: 476.6 ms, 256: 282.8 ms -> 256
 *   class 7 (larger): 32: 23420.0 ms, 64: 11914.3 ms, 128: 5882.1 ms, 256: 3470.7 ms -> 256
 */
#ifndef LGB_FACTOR_TUNE_H
#define LGB_FACTOR_TUNE_H
static const int lgb_factor_threads[LGB_NCLS] = {32, 32, 64, 256, 256, 256, 256, 256};
#endif
