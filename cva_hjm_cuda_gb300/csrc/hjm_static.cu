// hjm_static.cu -- hjm_run_static, the valuation entry point that allocates
// no device memory.
//
// Who needs it: a host that owns all device memory up front and forbids
// allocation afterwards -- a risk server whose pool allocator has already
// reserved the GPU, a pricing plugin loaded into such a process, or a
// latency-bound intraday loop that cannot afford the implicit device-wide
// synchronisation a cudaMalloc/cudaFree may cause.  Those callers cannot use
// hjm_run, whose context grows its buffers with cudaMalloc on demand.
//
// How: the only device memory the valuation needs besides the caller's
// inputs and outputs is the per-CTA partial sums of the path kernel, the
// column sums and the small result block.  Here they live in one file-scope
// __device__ array of fixed size (HJM_STATIC_MAX_PATHS paths), which every
// GPU that loads the library holds until the process exits.  Host code cannot
// use the array's name as a device address (it names a host-side stand-in),
// so the first call on each device looks the address up with
// cudaGetSymbolAddress, with that device current, and passes it to the same
// path and reduction kernels that hjm_run launches.
//
// A volatility table whose factors are quadratics in T (the synthetic
// factors of the configured workloads) runs the polynomial decomposition in
// both precisions, as hjm_run does.  FP64 runs take a response form whenever
// its table fits a second static array (4 MB; recomputed on the device at
// every call) and one launch covers the run's dates (hjm_run takes a response
// form for every FP64 valuation, in as many windows as it needs, each after
// the last with a carry): with polynomial factors the decomposition's
// remainder in double-FP32 impulse-response sums, else the whole stochastic
// curve as double-FP32 sums of the three factors' responses (12x the
// convected table step on the 10y swap).  Other FP64 runs take the convected
// step (decomposed or table).  Mixed precision with polynomial factors takes
// the FP32 response form where hjm_run does (its table, also rebuilt at every
// call, in the same static array), else the convected pairs.
//
// Limits: at most HJM_STATIC_MAX_PATHS paths per call; EE and CVA only (the
// per-path exposure store a PFE needs would not fit a modest static buffer).
// Every call shares the array: calls that overlap on the GPU (two streams, two
// host threads) race and must be serialised by the caller.  Nothing in the
// array has to start at zero (every element a call reads was written earlier
// in that call); the result block is cleared anyway.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/hjm_cva.h"
#include "hjm_eresp.h"
#include "hjm_kernels.h"

using namespace hjm;

namespace hjm {
void set_thread_error(const char* msg);  // hjm_capi.cu: the message hjm_last_error(NULL) returns
bool fit_quadratic_vols(const double* vol, int nt, double dtau, double* coef);  // hjm_capi.cu
bool fit_cubic_resid(const double* vol, int nt, double dtau, double* coef, int* degs, double* resid);  // hjm_capi.cu
void mixed_cubic_params(int nt, double dtau, double dt, int n_blocks, const double* cubic, MixedParams& M);  // hjm_capi.cu
}

namespace {

constexpr int kMinCta = 64;  // the smallest CTA of the path kernels (FP64)
constexpr int64_t kStaticCtas = (HJM_STATIC_MAX_PATHS + kMinCta - 1) / kMinCta;
constexpr int kStaticCols = kMaxTenor;                  // partial row: dates + 2 <= 64 doubles
constexpr size_t kPartialsDoubles = (size_t)kStaticCtas * kStaticCols;
constexpr size_t kSumsOffset = kPartialsDoubles;        // 2 * kMaxTenor doubles
constexpr size_t kResultOffset = kSumsOffset + 2 * kMaxTenor;
constexpr size_t kScratchDoubles = kResultOffset + kResLen;
constexpr size_t kStaticRespEntries = (size_t)1 << 18;  // double2: 4 MB of response table
constexpr int kMaxDevices = 64;

std::mutex g_static_mu;
double* g_static_ptr[kMaxDevices] = {};
double2* g_static_resp_ptr[kMaxDevices] = {};

hjm_status static_fail(hjm_status st, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    set_thread_error(buf);  // read back with hjm_last_error(NULL)
    return st;
}

}  // namespace

// The scratch: 8.4 MB of FP64 per device (HJM_STATIC_MAX_PATHS / 64 CTA rows
// of 64 partial sums, plus column sums and the result block).
static __device__ __align__(256) double g_hjm_static_scratch[kScratchDoubles];
// ... and 4 MB for the FP64 response table (the float4 entries of either
// response form, in a double2 array for its 16-byte alignment).
static __device__ __align__(256) double2 g_hjm_static_resp[kStaticRespEntries];
static_assert(sizeof(float4) == sizeof(double2), "both response tables use 16-byte entries");

#define STATIC_CUDA(call)                                                                          \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return static_fail(HJM_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));      \
    } while (0)

// Device addresses of the two static arrays on the current device, looked up
// once per device (the first call on a device does this; make that first call
// before any stream capture).
static hjm_status static_scratch(double** out, double2** resp_out)
{
    int dev = 0;
    STATIC_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) return static_fail(HJM_ERR_UNSUPPORTED, "device %d beyond %d", dev, kMaxDevices);
    std::lock_guard<std::mutex> lock(g_static_mu);
    if (!g_static_ptr[dev]) {
        void* p = nullptr;
        void* q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_hjm_static_scratch);
        if (e == cudaSuccess) e = cudaGetSymbolAddress(&q, g_hjm_static_resp);
        if (e != cudaSuccess || p == nullptr || q == nullptr)
            return static_fail(HJM_ERR_CUDA, "cudaGetSymbolAddress(scratch) on device %d failed: %s", dev,
                               cudaGetErrorString(e));
        g_static_resp_ptr[dev] = static_cast<double2*>(q);
        g_static_ptr[dev] = static_cast<double*>(p);
    }
    *out = g_static_ptr[dev];
    *resp_out = g_static_resp_ptr[dev];
    return HJM_OK;
}

// Host-side inputs of one call, in FP64: the same construction hjm_run uses
// (deterministic curve p and its discount integrals, per-date payoff vectors,
// CVA weights), restated here so that this entry point shares no state with
// the context-based one.
template <typename T>
static void static_params(int nt, double dtau, const double* spot, const double* vol, const double* drift,
                          const double* payA, const double* payB, int stride, int B, int64_t n_paths, double dt,
                          uint64_t seed, uint64_t path_offset, double hazard, double recovery, PathParams<T>& P,
                          FinalParams& F)
{
    std::memset(&P, 0, sizeof(P));
    std::memset(&F, 0, sizeof(F));
    const double sq = std::sqrt(dt);
    for (int k = 0; k < kFactors; ++k)
        for (int t = 0; t < nt; ++t) P.sv[k][t] = (T)(sq * vol[(size_t)k * nt + t]);
    double p[kMaxTenor], pn[kMaxTenor], acc[kMaxTenor];  // no heap use either
    for (int t = 0; t < nt; ++t) {
        p[t] = spot[t];
        acc[t] = 0.0;
    }
    for (int s = 0; s < stride; ++s)
        for (int t = 0; t < nt; ++t) acc[t] += p[t];
    P.psamp[1] = p[1];
    P.psum[1] = acc[1];
    for (int b = 1; b < B; ++b) {
        for (int s = 0; s < stride; ++s) {
            for (int t = 0; t < nt; ++t) {
                const double dF = (t == nt - 1) ? p[t] - p[t - 1] : p[t + 1] - p[t];
                double dfbar = drift[t] * dt;
                dfbar += (dF / dtau) * dt;
                pn[t] = p[t] + dfbar;
            }
            for (int t = 0; t < nt; ++t) {
                p[t] = pn[t];
                acc[t] += p[t];
            }
        }
        P.psamp[b + 1] = p[b + 1];
        P.psum[b + 1] = acc[b + 1];
    }
    for (int i = 0; i < nt; ++i) {
        P.payA[i] = payA[i];
        P.payB[i] = payB[i];
    }
    for (int j = 1; j <= B; ++j) {
        const double t0 = (j - 1) * dtau, t1 = j * dtau;
        const double e0 = std::exp(-hazard * t0), e1 = std::exp(-hazard * t1);
        P.cvaw[j] = (1.0 - recovery) * (e0 - e1);
        F.cvaw[j] = P.cvaw[j];
        F.dcvaw[j] = (1.0 - recovery) * (-t0 * e0 + t1 * e1);
    }
    P.c = (T)(dt / dtau);
    // c dtau and c dtau^2 rounded as hjm_run forms them (fill_params)
    P.k1 = (dt / dtau) * dtau;
    P.k2 = (dt / dtau) * dtau * dtau;
    fill_growth_scale(P, dt / dtau, P.k2, stride, B);
    for (int t = 0; t < nt; ++t) P.tau[t] = (T)(dtau * t);
    P.dt = dt;
    P.m = 1.0 / dtau;
    P.inv_m = dtau;
    P.key0 = (uint32_t)seed;
    P.key1 = (uint32_t)(seed >> 32);
    philox_round_keys(P.key0, P.key1, P.rk0, P.rk1);
    P.inv_c = dtau / dt;
    P.path_offset = path_offset;
    P.n_paths = n_paths;
    P.ld = 0;
    P.n_blocks = B;
    P.stride = stride;
    P.store_exposures = 0;
    F.n_paths = n_paths;
    F.n_blocks = B;
}

static bool all_finite(const double* a, size_t n)
{
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(a[i])) return false;
    return true;
}

hjm_status hjm_run_static(void* cuda_stream, int32_t n_tenor, double dtau, const double* spot_host,
                          const double* vol_host, const double* drift_host, double notional, double fixed_rate,
                          const double* accrual_host, int32_t payer, int64_t n_paths, int32_t n_steps, double dt,
                          uint64_t seed, uint64_t path_offset, int32_t precision, double hazard_rate,
                          double recovery, double* ee_out, double* cva_out)
{
    // ---- validation (nothing is allocated on any path) ----
    if (n_paths <= 0 || n_paths > HJM_STATIC_MAX_PATHS)
        return static_fail(HJM_ERR_INVALID_ARGUMENT,
                           "n_paths %lld outside [1, %d]: hjm_run_static serves at most HJM_STATIC_MAX_PATHS paths "
                           "per call (use hjm_run, or split the paths with path_offset)",
                           (long long)n_paths, (int)HJM_STATIC_MAX_PATHS);
    if (!path_tenor_supported(n_tenor))
        return static_fail(HJM_ERR_UNSUPPORTED, "n_tenor %d: path kernels are built for 51 and 61 tenors", n_tenor);
    if (!spot_host || !vol_host || !accrual_host || !ee_out || !cva_out)
        return static_fail(HJM_ERR_INVALID_ARGUMENT, "spot, vol, accrual, ee_out and cva_out must not be null");
    if (!(dtau > 0.0) || !(dt > 0.0) || !std::isfinite(dtau) || !std::isfinite(dt))
        return static_fail(HJM_ERR_INVALID_ARGUMENT, "dtau and dt must be finite and > 0");
    if (precision != HJM_PRECISION_FP64 && precision != HJM_PRECISION_MIXED)
        return static_fail(HJM_ERR_INVALID_ARGUMENT, "unknown precision %d", precision);
    if (!(hazard_rate >= 0.0) || !std::isfinite(hazard_rate) || !(recovery >= 0.0 && recovery <= 1.0))
        return static_fail(HJM_ERR_INVALID_ARGUMENT, "hazard must be >= 0 and recovery in [0, 1]");
    if (!all_finite(spot_host, n_tenor) || !all_finite(vol_host, (size_t)HJM_N_FACTOR * n_tenor) ||
        !all_finite(accrual_host, n_tenor) || (drift_host && !all_finite(drift_host, n_tenor)) ||
        !std::isfinite(notional) || !std::isfinite(fixed_rate))
        return static_fail(HJM_ERR_INVALID_ARGUMENT, "inputs must be finite");
    const double r = dtau / dt;
    const long stride = std::lround(r);
    if (stride < 1 || std::fabs(r - (double)stride) > 1e-9 * r)
        return static_fail(HJM_ERR_INVALID_ARGUMENT, "dtau/dt = %.17g is not an integer number of steps", r);
    if (stride < 2)
        return static_fail(HJM_ERR_UNSUPPORTED, "dt must be at most dtau/2 (the kernels need c = dt/dtau < 1)");
    if (precision == HJM_PRECISION_MIXED && (double)n_steps * std::log1p(1.0 / ((double)stride - 1.0)) > 80.0)
        return static_fail(HJM_ERR_UNSUPPORTED,
                           "mixed precision: the growth-scaled curve would exceed e^80; use FP64 or a smaller dt");
    if (n_steps <= 0 || n_steps % stride != 0)
        return static_fail(HJM_ERR_INVALID_ARGUMENT, "n_steps %d is not a positive multiple of %ld", n_steps, stride);
    const int B = n_steps / (int)stride;
    if (B > n_tenor - 1)
        return static_fail(HJM_ERR_INVALID_ARGUMENT, "%d sampled dates need %d tenors; the grid has %d", B, B + 1,
                           n_tenor);
    const int R = B + 3;
    // quadratic factors: the polynomial decomposition's coefficients
    // sqrt(dt) c_{k,d}, as hjm_run's fill_params
    double coef[HJM_N_VOL_COEF];
    const bool poly = fit_quadratic_vols(vol_host, n_tenor, dtau, coef);
    // a table that is a cubic up to a small residual (the reference's own PCA
    // table): FP64 the response form with the residual, mixed precision the
    // cubic polynomial form, as hjm_run
    double cubic[HJM_N_FACTOR * 4], resid[HJM_N_FACTOR * HJM_MAX_TENOR];
    int cdegs[HJM_N_FACTOR];
    const bool cub = !poly && fit_cubic_resid(vol_host, n_tenor, dtau, cubic, cdegs, resid);
    // mixed precision with polynomial factors: the response form when the
    // dates its remainder reaches fit its slots and its table the static array
    const int mresp_ns =
        (precision == HJM_PRECISION_MIXED && (poly || cub)) ? mresp_slots(n_tenor, dt / dtau, dtau, (int)stride, B) : 0;
    const bool mresp = mresp_ns > 0 && mresp_table_elems((int)stride, B, mresp_ns) <= kStaticRespEntries;
    const int cta = mresp ? kCta : path_cta(precision == HJM_PRECISION_MIXED, n_tenor, B, poly || cub);
    const int64_t n_ctas = (n_paths + cta - 1) / cta;
    if (R > kStaticCols || n_ctas > kStaticCtas)
        return static_fail(HJM_ERR_INVALID_ARGUMENT, "run exceeds the static scratch");

    // ---- host-side inputs ----
    double drift[HJM_MAX_TENOR], payA[HJM_MAX_TENOR], payB[HJM_MAX_TENOR];
    if (drift_host) {
        for (int t = 0; t < n_tenor; ++t) drift[t] = drift_host[t];
    } else {
        for (int t = 0; t < n_tenor; ++t) drift[t] = 0.0;
        for (int k = 0; k < HJM_N_FACTOR; ++k) {
            const double* s = vol_host + (size_t)k * n_tenor;
            double integral = 0.0;
            for (int i = 0; i < n_tenor; ++i) {
                if (i > 0) integral += 0.5 * (s[i] + s[i - 1]) * dtau;
                drift[i] += s[i] * integral;
            }
        }
    }
    const double sign = payer ? 1.0 : -1.0;
    for (int i = 0; i < n_tenor; ++i) {
        payA[i] = sign * notional * accrual_host[i];
        payB[i] = sign * notional * accrual_host[i] * fixed_rate;
    }

    double* scratch = nullptr;
    double2* resp_table = nullptr;
    hjm_status st = static_scratch(&scratch, &resp_table);
    if (st != HJM_OK) return st;
    double* partials = scratch;
    double* sums = scratch + kSumsOffset;
    double* result = scratch + kResultOffset;
    const cudaStream_t s = (cudaStream_t)cuda_stream;

    STATIC_CUDA(cudaMemsetAsync(result, 0, sizeof(double) * kResLen, s));
    FinalParams F;
    const double sq = std::sqrt(dt);
    if (precision == HJM_PRECISION_MIXED) {
        PathParams<float> P;
        static_params<float>(n_tenor, dtau, spot_host, vol_host, drift, payA, payB, (int)stride, B, n_paths, dt, seed,
                             path_offset, hazard_rate, recovery, P, F);
        if (poly)
            for (int k = 0; k < kFactors; ++k)
                for (int d = 0; d < 3; ++d) P.svc[k][d] = sq * coef[k * 3 + d];
        MixedParams M;
        pack_mixed_params(n_tenor, P, M);
        if (cub) mixed_cubic_params(n_tenor, dtau, dt, B, cubic, M);
        if (mresp) {
            float4* table = reinterpret_cast<float4*>(resp_table);
            STATIC_CUDA(launch_mresp_table(n_tenor, dt / dtau, dtau, (int)stride, B, mresp_ns, false, table, s));
            STATIC_CUDA(launch_path_mixed_resp(M, mresp_ns, cub, table, nullptr, partials, nullptr, s));
        } else {
            STATIC_CUDA(launch_path_mixed(n_tenor, M, poly, nullptr, partials, nullptr, s, cub));
        }
    } else {
        PathParams<double> P;
        static_params<double>(n_tenor, dtau, spot_host, vol_host, drift, payA, payB, (int)stride, B, n_paths, dt,
                              seed, path_offset, hazard_rate, recovery, P, F);
        if (poly)
            for (int k = 0; k < kFactors; ++k)
                for (int d = 0; d < 3; ++d) P.svc[k][d] = sq * coef[k * 3 + d];
        const size_t entries = response_table_vol_elems((int)stride, B);
        const int nres = cub ? eresp_residual_factors(resid, vol_host, n_tenor) : 0;
        const int first = (poly || cub) ? eresp_first_active_date(n_tenor, dt / dtau, (int)stride, B, nres) : 2;
        if ((poly || cub) && eresp_windows(B, first, nullptr, nullptr, nullptr, eresp_window_dates(nres)) == 1 &&
            eresp_table_elems((int)stride, B, cub ? 4 : 3, nres, 1) <= kStaticRespEntries) {
            // the decomposition's response form in one window: its table (FP32
            // pairs, 16 bytes per entry) in the static array
            EulerRespFrame fr;
            int degs;
            eresp_make_frame(dt, dtau, n_tenor, P.svc, cub ? cubic : nullptr, cdegs, eresp_window_centre(dtau, 1, B), fr,
                             degs);
            for (int i = 0; i < HJM_N_FACTOR * n_tenor; ++i) resid[i] *= sq;
            float4* table = reinterpret_cast<float4*>(resp_table);
            STATIC_CUDA(launch_eresp_tables(n_tenor, dt / dtau, dtau, (int)stride, B, &fr, 1, cub ? resid : nullptr, nres,
                                            false, table, s));
            EulerRespParams E;
            std::memset(&E, 0, sizeof(E));
            E.P = P;
            E.frame = block_frame_n(fr.n, (int)stride);
            E.row = eresp_row(B);
            E.renorm = (cub || B > kRespSlots + 1) ? 1 : 0;  // as hjm_run
            STATIC_CUDA(launch_path_fp64_eresp(E, &fr, degs, nres, table, first, nullptr, partials, nullptr, nullptr, s,
                                               nullptr));
        } else if (B >= 2 && B <= response_max_dates() && entries <= kStaticRespEntries) {
            // the response form: its table (zero outside the live entries) into the static array
            STATIC_CUDA(cudaMemsetAsync(resp_table, 0, sizeof(float4) * entries, s));
            float4* vtable = reinterpret_cast<float4*>(resp_table);
            STATIC_CUDA(launch_response_table_vol(n_tenor, dt / dtau, (int)stride, B, false, &P.sv[0][0], vtable, s));
            // one launch of 24 slots (the static scratch holds no carry)
            STATIC_CUDA(launch_path_fp64_vresp(n_tenor, P, vtable, nullptr, partials, nullptr, nullptr, s, nullptr, 24));
        } else {
            STATIC_CUDA(launch_path_fp64(n_tenor, P, poly, nullptr, partials, nullptr, s));
        }
    }
    STATIC_CUDA(launch_reduce(partials, n_ctas, R, sums, F, result, s));
    double res[kResLen];
    STATIC_CUDA(cudaMemcpyAsync(res, result, sizeof(res), cudaMemcpyDeviceToHost, s));
    STATIC_CUDA(cudaStreamSynchronize(s));
    for (int j = 0; j < n_tenor; ++j) ee_out[j] = res[kResEE + j];
    cva_out[HJM_CVA_VALUE] = res[kResCVA];
    cva_out[HJM_CVA_STDERR] = res[kResCVAStderr];
    cva_out[HJM_CVA_DHAZARD] = res[kResDCVADHazard];
    return HJM_OK;
}
