// hjm_dropin.cpp -- the reference's two GPU entry points on top of the C ABI.
//
// calculateExposureMultiGPU(double*, InterestRateSwap<double>, ...) and its
// float overload (simulation_gpu.h:12,14; simulation_gpu.cu:1243-1250) keep
// their signatures, argument meaning and print-and-continue error behaviour;
// the body is one hjm_run on a process-wide context.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <vector>

#include "../../include/hjm_cva.h"
#include "../../include/hjm_dropin.h"

namespace {

constexpr int kTimepoints = 51;   // TIMEPOINTS, simulation_gpu.cu:33
constexpr uint64_t kSeed = 1234;  // simulation_gpu.cu:963

std::mutex g_mu;
hjm_ctx* g_ctx = nullptr;

template <typename real>
void run_dropin(real* expected_exposure, const InterestRateSwap<real>& payOff, const real* accrual,
                const real* spot_rates, const real* drift, const real* volatilities, int num_gpus, int simN, real dt,
                int32_t precision)
{
    if (!expected_exposure) {
        std::fprintf(stderr, "ERROR: calculateExposureMultiGPU: expected_exposure is null\n");
        return;
    }
    std::memset(expected_exposure, 0, kTimepoints * sizeof(real));
    if (!accrual || !spot_rates || !drift || !volatilities) {
        std::fprintf(stderr, "ERROR: calculateExposureMultiGPU: null input array\n");
        return;
    }
    if (num_gpus != 1)
        std::fprintf(stderr, "calculateExposureMultiGPU: num_gpus=%d requested; this engine runs all %d paths on one GPU\n",
                     num_gpus, simN);
    std::vector<double> acc(kTimepoints), spot(kTimepoints), mu(kTimepoints), vol(3 * kTimepoints);
    for (int t = 0; t < kTimepoints; ++t) {
        acc[t] = accrual[t];
        spot[t] = spot_rates[t];
        mu[t] = drift[t];
    }
    for (int t = 0; t < 3 * kTimepoints; ++t) vol[t] = volatilities[t];
    // Step counts are ratios of the caller's reals, rounded to the nearest
    // integer when within the reals' rounding of one (relative 1e-9 for
    // double, 1e-6 for float: 0.5f / 0.01f is 50.0000011 in double).  A float
    // dt is then taken as dtau / stride exactly, the step the caller meant
    // (the reference's float path computes (int)(dtau/dt) = 50 in float).
    const double tol = sizeof(real) == sizeof(float) ? 1e-6 : 1e-9;
    double ddt = (double)dt;
    if (sizeof(real) == sizeof(float) && ddt > 0.0) {
        const double r = (double)payOff.dtau / ddt;
        const long rs = std::lround(r);
        if (rs >= 1 && std::fabs(r - (double)rs) <= tol * r) ddt = (double)payOff.dtau / (double)rs;
    }
    // pathN = expiry / dt (simulation_gpu.cu:959)
    const double ratio = (double)payOff.expiry / ddt;
    const long rn = std::lround(ratio);
    const int n_steps = (std::fabs(ratio - (double)rn) <= tol * ratio) ? (int)rn : (int)ratio;

    std::lock_guard<std::mutex> lock(g_mu);
    hjm_status st = HJM_OK;
    if (!g_ctx) st = hjm_ctx_create(0, &g_ctx);
    if (st != HJM_OK) {
        std::fprintf(stderr, "ERROR: calculateExposureMultiGPU: %s\n", hjm_last_error(nullptr));
        g_ctx = nullptr;
        return;
    }
    std::vector<double> ee(kTimepoints, 0.0);
    st = hjm_set_market(g_ctx, kTimepoints, (double)payOff.dtau, spot.data(), vol.data(), 3, mu.data());
    if (st == HJM_OK) st = hjm_set_swap(g_ctx, (double)payOff.notional, (double)payOff.K, acc.data(), 1);
    if (st == HJM_OK)
        st = hjm_run(g_ctx, simN, n_steps, ddt, kSeed, 0, precision, 0.0, 0.0, 0.0, ee.data(), nullptr, nullptr);
    if (st != HJM_OK) {
        std::fprintf(stderr, "ERROR: calculateExposureMultiGPU: %s\n", hjm_last_error(g_ctx));
        return;
    }
    for (int t = 0; t < kTimepoints; ++t) expected_exposure[t] = (real)ee[t];
}

}  // namespace

void calculateExposureMultiGPU(double* expected_exposure, InterestRateSwap<double> payOff, double* accrual,
                               double* spot_rates, double* drift, double* volatilities, double scale, int num_gpus,
                               int simN, double dt)
{
    (void)scale;  // parsed and unused by the reference as well
    run_dropin<double>(expected_exposure, payOff, accrual, spot_rates, drift, volatilities, num_gpus, simN, dt,
                       HJM_PRECISION_FP64);
}

void calculateExposureMultiGPU(float* expected_exposure, InterestRateSwap<float> payOff, float* accrual,
                               float* spot_rates, float* drifts, float* volatilities, float scale, const int num_gpus,
                               int scenarios, float dt)
{
    (void)scale;
    run_dropin<float>(expected_exposure, payOff, accrual, spot_rates, drifts, volatilities, num_gpus, scenarios, dt,
                      HJM_PRECISION_MIXED);
}

// C entry for bindings that cannot call C++ (ctypes in the tests): the double
// overload with the swap passed as its scalars.
extern "C" void hjm_dropin_calculate_exposure_fp64(double* expected_exposure, double notional, double K, double expiry,
                                                   double dtau, double* accrual, double* spot_rates, double* drift,
                                                   double* volatilities, int num_gpus, int simN, double dt)
{
    InterestRateSwap<double> sw(nullptr, nullptr, nullptr, notional, K, expiry, dtau);
    calculateExposureMultiGPU(expected_exposure, sw, accrual, spot_rates, drift, volatilities, 0.0, num_gpus, simN, dt);
}

extern "C" void hjm_dropin_calculate_exposure_fp32(float* expected_exposure, float notional, float K, float expiry,
                                                   float dtau, float* accrual, float* spot_rates, float* drift,
                                                   float* volatilities, int num_gpus, int simN, float dt)
{
    InterestRateSwap<float> sw(nullptr, nullptr, nullptr, notional, K, expiry, dtau);
    calculateExposureMultiGPU(expected_exposure, sw, accrual, spot_rates, drift, volatilities, 0.0f, num_gpus, simN, dt);
}
