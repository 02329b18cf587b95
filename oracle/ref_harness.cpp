/*
 * ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
 *
 * Compiles the reference's own CPU path (simulation_cpu.h, included from the
 * read-only reference tree by the Makefile in this folder; nothing of it is
 * copied here) into oracle/_ref/libhjm_ref.so, and exposes two C entry points
 * that tests and the golden-vector generator call through ctypes:
 *
 *   ref_exposure_paths  -- the reference's per-path functions
 *                          __generatePaths_kernel_cpu (simulation_cpu.h:188),
 *                          __calculateExposure_kernel (:270) and
 *                          __calculateExpectedExposure_kernel (:336), driven by
 *                          a loop that mirrors calculateExposureCPU (:405-458)
 *                          but takes the normals from the caller and zeroes
 *                          the numeraires first (the reference leaves the ones
 *                          no block writes uninitialised);
 *   ref_calculate_exposure_cpu -- the reference's whole, unmodified
 *                          calculateExposureCPU<double> (:350), which draws
 *                          its own cuRAND host XORWOW normals (seed 1234).
 *
 * The reference fixes the tenor count at 51 (_TIMEPOINTS), so both entry
 * points accept 51 tenors only.
 */
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>
#include <cstring>
#include <utility>

/* the reference relies on <cmath>/<cstdio> arriving through other headers */
#include "simulation_cpu.h"

extern "C" int ref_exposure_paths(int n_steps, const double* spot, const double* vol,
                                  const double* drift, const double* accrual, double notional,
                                  double strike, int n_paths, const double* normals,
                                  double* exposures /* [n_paths][51] */, double* ee /* [51] */)
{
    const int T = _TIMEPOINTS;
    const int stride = 50;  /* dtau / dt with the reference's defaults 0.5 / 0.01 */
    if (n_steps % stride != 0 || n_steps / stride > T - 1) return -1;

    std::vector<__real2<double>> numeraires((size_t)n_paths * T);
    std::memset(numeraires.data(), 0, sizeof(__real2<double>) * numeraires.size());
    /* one extra element: __calculateExposure_kernel writes exposure[51] */
    std::vector<double> x((size_t)n_paths * T + 1, 0.0);
    std::vector<double> r0((size_t)n_paths * T, 0.0), r1((size_t)n_paths * T, 0.0), acc((size_t)n_paths * T, 0.0);
    double* simulated_rates = r0.data();
    double* simulated_rates0 = r1.data();

    for (int path = 0; path < n_steps; path += stride) {
        for (int s = 0; s < n_paths; ++s) {
            __generatePaths_kernel_cpu(&numeraires[(size_t)s * T], T, const_cast<double*>(drift),
                                       const_cast<double*>(vol),
                                       const_cast<double*>(normals) + (size_t)s * n_steps * 3,
                                       const_cast<double*>(spot), &simulated_rates[(size_t)s * T],
                                       &simulated_rates0[(size_t)s * T], &acc[(size_t)s * T],
                                       n_steps, path);
        }
        std::swap(simulated_rates, simulated_rates0);
    }
    for (int s = 0; s < n_paths; ++s)
        __calculateExposure_kernel(&x[(size_t)s * T], &numeraires[(size_t)s * T], notional, strike,
                                   const_cast<double*>(accrual), n_paths);

    std::vector<double> ones((size_t)n_paths, 1.0), y((size_t)T, 0.0);
    __calculateExpectedExposure_kernel(ee, x.data(), ones.data(), y.data(), n_paths);
    std::memcpy(exposures, x.data(), sizeof(double) * (size_t)n_paths * T);
    return 0;
}

extern "C" int ref_calculate_exposure_cpu(double* ee /* [51] */, double notional, double strike,
                                          double expiry, double dtau, const double* accrual,
                                          const double* spot, const double* drift, const double* vol,
                                          int n_paths, double dt)
{
    InterestRateSwap<double> swap(nullptr, nullptr, nullptr, notional, strike, expiry, dtau);
    calculateExposureCPU<double>(ee, swap, const_cast<double*>(accrual), const_cast<double*>(spot),
                                 const_cast<double*>(drift), const_cast<double*>(vol), n_paths, dt);
    return 0;
}
