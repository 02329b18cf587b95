// dropin_caller.cpp -- a C++ caller of the drop-in entry points, built by the
// tests with g++ against include/hjm_dropin.h and libhjmcva.so.
//
// It calls calculateExposureMultiGPU the way the reference's driver does
// (simulation_gpu_testing.cpp:195-216): the swap built as
// InterestRateSwap<real>(schedule, schedule, schedule, notional, K, expiry,
// dtau), its InterestRateSwap_D twin constructed beside it, host arrays for
// accrual, spot, drift and the factor-major volatility table.  Both overloads
// run on the same inputs (the float one on the inputs rounded to float).
//
//   dropin_caller <inputs.bin> <outputs.bin> <paths> <num_gpus> <dt>
//
// inputs.bin: 51 spot, 153 vol, 51 drift, 51 accrual, then notional, K,
// expiry, dtau (doubles).  outputs.bin: the 51 EE values of the double
// overload, then those of the float overload (widened), as doubles.  The
// outputs are filled with NaN before each call, so every value written is
// the call's own.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "hjm_dropin.h"

int main(int argc, char** argv)
{
    if (argc != 6) {
        std::fprintf(stderr, "usage: %s inputs.bin outputs.bin paths num_gpus dt\n", argv[0]);
        return 2;
    }
    const int n_paths = std::atoi(argv[3]);
    const int num_gpus = std::atoi(argv[4]);
    const double dt = std::atof(argv[5]);
    constexpr int T = 51;
    std::vector<double> in(4 * T + 2 * T + 4);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f) return 3;
    const size_t n_in = std::fread(in.data(), sizeof(double), 6 * T + 4, f);
    std::fclose(f);
    if (n_in != 6 * T + 4) return 3;
    double* spot = in.data();
    double* vol = spot + T;
    double* drift = vol + 3 * T;
    double* accrual = drift + T;
    const double notional = accrual[T], K = accrual[T + 1], expiry = accrual[T + 2], dtau = accrual[T + 3];

    std::vector<double> schedule(T);
    for (int t = 0; t < T; ++t) schedule[t] = dtau * t;
    std::vector<float> schedule_f(schedule.begin(), schedule.end());

    InterestRateSwap<double> payOff(&schedule[0], &schedule[0], &schedule[0], notional, K, expiry, dtau);
    InterestRateSwap_D payOff_d(&schedule[0], &schedule[0], &schedule[0], notional, K, expiry, dtau);
    InterestRateSwap<float> payOff_f(&schedule_f[0], &schedule_f[0], &schedule_f[0], (float)notional, (float)K,
                                     (float)expiry, (float)dtau);
    if (payOff_d.notional != payOff.notional || payOff_d.expiry != payOff.expiry || payOff_d.dtau != payOff.dtau)
        return 4;

    std::vector<double> ee(T, std::nan(""));
    calculateExposureMultiGPU(&ee[0], payOff, accrual, spot, drift, vol, 0.0, num_gpus, n_paths, dt);

    std::vector<float> spot_f(spot, spot + T), vol_f(vol, vol + 3 * T), drift_f(drift, drift + T),
        accrual_f(accrual, accrual + T);
    std::vector<float> ee_f(T, std::nanf(""));
    calculateExposureMultiGPU(&ee_f[0], payOff_f, &accrual_f[0], &spot_f[0], &drift_f[0], &vol_f[0], 0.0f, num_gpus,
                              n_paths, (float)dt);

    std::vector<double> out(2 * T);
    for (int t = 0; t < T; ++t) {
        out[t] = ee[t];
        out[T + t] = (double)ee_f[t];
    }
    f = std::fopen(argv[2], "wb");
    if (!f) return 5;
    const size_t n_out = std::fwrite(out.data(), sizeof(double), out.size(), f);
    std::fclose(f);
    return n_out == out.size() ? 0 : 5;
}
