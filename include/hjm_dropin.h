/*
 * hjm_dropin.h -- drop-in replacement for the reference's GPU entry points.
 *
 * Declares exactly the two overloads of mahsanchez/cva_hjm_cuda
 * simulation_gpu.h:12 and :14 (defined at simulation_gpu.cu:1243 and :1248).
 * Link libhjmcva.so instead of the reference's simulation_gpu.cu object; the
 * call, its arguments and its output are unchanged:
 *
 *   expected_exposure  [51] out: EE on the 0.5y tenor grid, mean over simN paths
 *   payOff             notional, K, dtau, expiry (schedules unused, as before)
 *   accrual, spot_rates, drift  [51] host arrays; volatilities [3 * 51] factor-major
 *   scale              unused (the reference parses and ignores it)
 *   num_gpus           the engine runs on one GPU; other values print a note
 *   simN               number of Monte Carlo paths
 *   dt                 Euler step; expiry / dt steps in blocks of dtau / dt
 *
 * The double overload runs the FP64 path; the float overload runs the mixed
 * precision path (FP32 curve and pricing, FP64 discount accumulation and
 * reductions).  Normals are Philox4x32-10 with the reference's seed 1234
 * (simulation_gpu.cu:963) instead of the reference's cuRAND XORWOW buffer.
 * Errors are printed to stderr and the output is zero-filled, as the
 * reference prints and continues (simulation_gpu.cu:71-106, :1156).
 * Unlike the reference, the call is re-entrant: it serialises on an internal
 * context instead of writing global __constant__ symbols.
 */
#ifndef HJM_DROPIN_H
#define HJM_DROPIN_H

#include "hjm_product.h"

void calculateExposureMultiGPU(double* expected_exposure, InterestRateSwap<double> payOff, double* accrual,
                               double* spot_rates, double* drift, double* volatilities, double scale, int num_gpus,
                               int simN, double dt);

void calculateExposureMultiGPU(float* expected_exposure, InterestRateSwap<float> payOff, float* accrual,
                               float* spot_rates, float* drifts, float* volatilities, float scale,
                               const int num_gpus, int scenarios, float dt);

/* C-callable forms of the two overloads (for bindings that cannot call C++,
 * e.g. ctypes): the swap is passed as its scalars, the schedules being unused. */
#ifdef __cplusplus
extern "C" {
#endif
void hjm_dropin_calculate_exposure_fp64(double* expected_exposure, double notional, double K, double expiry,
                                        double dtau, double* accrual, double* spot_rates, double* drift,
                                        double* volatilities, int num_gpus, int simN, double dt);
void hjm_dropin_calculate_exposure_fp32(float* expected_exposure, float notional, float K, float expiry,
                                        float dtau, float* accrual, float* spot_rates, float* drift,
                                        float* volatilities, int num_gpus, int simN, float dt);
#ifdef __cplusplus
}
#endif

#endif
