// hjm_capi.cu -- the C ABI of libhjmcva.so (declared in include/hjm_cva.h).
//
// Host orchestration that replaces __calculateExposureMultiGPU
// (simulation_gpu.cu:956-1241): instead of eight cudaMallocs, a cuRAND buffer,
// 2,500 launches with a device synchronisation after each and a host-side
// reduction, one context keeps grow-only device buffers, and one valuation is
// a fixed sequence of launches on one stream (path kernel, column reduction,
// finalisation, optional PFE selection) followed by one small copy-out.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/hjm_cva.h"
#include "hjm_eresp.h"
#include "hjm_kernels.h"

using namespace hjm;

namespace {

thread_local std::string g_thread_error;

// Device bytes a context's buffers hold, and the cap a caller may set on them
// (hjm_ctx_set_memory_limit; 0 = none).
struct MemBudget {
    size_t limit = 0;
    size_t used = 0;
};

struct DevBuf {
    void* p = nullptr;
    size_t bytes = 0;
    MemBudget* budget = nullptr;
    // Grow to at least need bytes (contents not kept).  A growth past the
    // budget's cap fails as an allocation failure would, before anything is
    // freed, so the buffer and the context stay as they were.
    cudaError_t ensure(size_t need)
    {
        if (need <= bytes) return cudaSuccess;
        if (budget && budget->limit && budget->used - bytes + need > budget->limit) return cudaErrorMemoryAllocation;
        release();
        cudaError_t e = cudaMalloc(&p, need);
        if (e == cudaSuccess) {
            bytes = need;
            if (budget) budget->used += need;
        } else {
            p = nullptr;
        }
        return e;
    }
    void release()
    {
        if (p) cudaFree(p);
        if (budget) budget->used -= bytes;
        p = nullptr;
        bytes = 0;
    }
};

}  // namespace

namespace hjm {
// Lets the allocation-free entry point (hjm_static.cu) report a failure
// through hjm_last_error(NULL); internal to the library.
__attribute__((visibility("hidden"))) void set_thread_error(const char* msg) { g_thread_error = msg; }
}  // namespace hjm

struct hjm_ctx {
    int device = 0;
    int n_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    std::string err;

    // market
    bool have_market = false;
    bool have_poly = false;       // coefficients given by hjm_set_market_poly (sensitivities)
    bool poly_path = false;       // the kernels run the polynomial decomposition (coef)
    bool allow_poly_path = true;  // hjm_ctx_set_vol_decomposition
    // cubic factors up to a small residual table (a PCA table printed to a
    // few decimals): the FP64 Euler response form's decomposition
    bool cubic_path = false;
    double cubic[HJM_N_FACTOR][4] = {};  // coefficients of (T - T_L)^d
    int cubic_degs[HJM_N_FACTOR] = {};
    std::vector<double> resid;            // [3][nt] sigma_k - cubic_k (unscaled)
    int scheme = HJM_SCHEME_EULER;  // hjm_ctx_set_scheme
    int remainder = HJM_REMAINDER_AUTO;  // hjm_ctx_set_remainder_form
    int nt = 0;
    double dtau = 0.5;
    std::vector<double> spot, vol, drift;
    double coef[HJM_N_VOL_COEF] = {0};

    // product: cash flow of date i = D_i * (payA[i] * L_i - payB[i])
    bool have_product = false;
    std::vector<double> payA, payB;

    bool keep_exposures = false;

    // device buffers
    DevBuf partials, sums, result, estore, sel, hist, ext, ext_raw, wide, scratch, ck_h, ck_a, vresp, eresp, carry,
        mresp;
    MemBudget budget;
    hjm_ctx()
    {
        for (DevBuf* b : buffers()) b->budget = &budget;
    }
    std::array<DevBuf*, 16> buffers()
    {
        return {&partials, &sums, &result, &estore, &sel, &hist, &ext, &ext_raw, &wide, &scratch, &ck_h, &ck_a,
                &vresp, &eresp, &carry, &mresp};
    }
    // the response tables in eresp, vresp and mresp hold the run shapes of
    // their keys; resp_used is recorded after the last kernel that reads one
    struct ErespKey {  // the response form's table in eresp (Euler or predictor-corrector)
        bool valid = false, pc = false;
        int nt = 0, stride = 0, B = 0, np = 0, nres = 0;
        double c = 0, dtau = 0;
        std::vector<EulerRespFrame> frames;  // one per window
        std::vector<double> resid;  // sqrt(dt)-scaled, empty without a residual
    } eresp_key;
    struct ErespFirst {  // eresp_first_active_date of the last run shape
        bool valid = false, pc = false;
        int nt = 0, stride = 0, B = 0, nres = 0;
        double c = 0;
        int first = 2;
    } eresp_first;
    struct VrespKey {  // the volatility-table response table in vresp
        bool valid = false;
        int nt = 0, stride = 0, B = 0, scheme = 0;
        double c = 0;
        std::vector<double> sv;
    } vresp_key;
    struct MrespKey {  // the mixed-precision response form's slots and its table in mresp
        bool valid = false, on_device = false, pc = false;
        int nt = 0, stride = 0, B = 0, ns = 0;
        double c = 0, dtau = 0;
    } mresp_key;
    cudaEvent_t resp_used = nullptr;

    // last valuation
    bool have_result = false;
    int64_t last_n_paths = 0;
    int last_n_dates = 0;
    bool last_mixed = false;
    bool last_stored = false;
    bool last_pfe = false;
    int64_t last_ld = 0;
    int64_t stat_launches = 0, stat_h2d = 0, stat_d2h = 0;
    // ring of event quadruples, one per valuation: before the path kernel,
    // after it, after the reductions, after the PFE selection
    static constexpr int kRing = 64;
    cudaEvent_t ring[kRing][4] = {};
    int64_t n_enqueued = 0;
    cudaEvent_t* ev = nullptr;  // the quadruple of the current valuation

    // what hjm_write_report writes: the last valuation fetched, or the last
    // adjoint run (run = the inputs of the call, filled at enqueue time)
    struct Report {
        bool valid = false, adjoint = false, pfe = false, external_normals = false;
        int64_t n_paths = 0;
        int n_steps = 0, n_dates = 0, precision = 0, vol_form = 0, ckpt = 0, nt = 0, scheme = 0;
        int remainder = 0;  // 1 convected, 2 impulse responses (0: not a valuation)
        double dt = 0, dtau = 0, hazard = 0, recovery = 0, pfe_q = 0;
        uint64_t seed = 0, path_offset = 0;
        std::vector<double> ee, pfe_v, dspot, ddrift;
        std::vector<double> levels;  // multi-level MC: [level][4] as hjm_run_mlmc's level_out
        double dcoef[HJM_N_VOL_COEF] = {0};
        bool have_dcoef = false;
        double cva = 0, cva_stderr = 0, dhazard = 0;
    } rep, rep_run;
};

static hjm_status fail(hjm_ctx* ctx, hjm_status st, const char* fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    if (ctx)
        ctx->err = buf;
    else
        g_thread_error = buf;
    return st;
}

#define HJM_CUDA(ctx, call)                                                                                 \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess)                                                                              \
            return fail((ctx), e_ == cudaErrorMemoryAllocation ? HJM_ERR_OUT_OF_MEMORY : HJM_ERR_CUDA,      \
                        "%s failed: %s", #call, cudaGetErrorString(e_));                                    \
    } while (0)

#define HJM_CHECK_CTX(ctx)                                                                                  \
    do {                                                                                                    \
        if (!(ctx)) return fail(nullptr, HJM_ERR_INVALID_ARGUMENT, "null context");                        \
    } while (0)

static bool finite_all(const double* a, size_t n)
{
    for (size_t i = 0; i < n; ++i)
        if (!std::isfinite(a[i])) return false;
    return true;
}

// Every hjm_* function below is declared extern "C" in hjm_cva.h, so its
// definition has C linkage.
const char* hjm_version(void) { return "hjmcva 0.1.0 (sm_103a)"; }

const char* hjm_last_error(const hjm_ctx* ctx) { return ctx ? ctx->err.c_str() : g_thread_error.c_str(); }

hjm_status hjm_ctx_create(int device, hjm_ctx** out)
{
    if (!out) return fail(nullptr, HJM_ERR_INVALID_ARGUMENT, "out is null");
    *out = nullptr;
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess || n <= 0)
        return fail(nullptr, HJM_ERR_NO_DEVICE, "no CUDA device: %s", cudaGetErrorString(e));
    if (device < 0 || device >= n)
        return fail(nullptr, HJM_ERR_INVALID_ARGUMENT, "device %d out of range [0, %d)", device, n);
    e = cudaSetDevice(device);
    if (e != cudaSuccess) return fail(nullptr, HJM_ERR_CUDA, "cudaSetDevice(%d): %s", device, cudaGetErrorString(e));
    cudaDeviceProp prop;
    e = cudaGetDeviceProperties(&prop, device);
    if (e != cudaSuccess) return fail(nullptr, HJM_ERR_CUDA, "cudaGetDeviceProperties: %s", cudaGetErrorString(e));
    if (prop.major < 10)
        return fail(nullptr, HJM_ERR_UNSUPPORTED, "device %d is sm_%d%d; this library is built for sm_103a", device,
                    prop.major, prop.minor);
    hjm_ctx* c = new hjm_ctx();
    c->device = device;
    c->n_sms = prop.multiProcessorCount;
    e = cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete c;
        return fail(nullptr, HJM_ERR_CUDA, "cudaStreamCreate: %s", cudaGetErrorString(e));
    }
    c->stream = c->own_stream;
    for (auto& q : c->ring)
        for (auto& ev : q) {
            e = cudaEventCreate(&ev);
            if (e != cudaSuccess) {
                hjm_ctx_destroy(c);
                return fail(nullptr, HJM_ERR_CUDA, "cudaEventCreate: %s", cudaGetErrorString(e));
            }
        }
    c->ev = c->ring[0];
    *out = c;
    return HJM_OK;
}

hjm_status hjm_ctx_destroy(hjm_ctx* ctx)
{
    if (!ctx) return HJM_OK;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (DevBuf* b : ctx->buffers()) b->release();
    if (ctx->resp_used) cudaEventDestroy(ctx->resp_used);
    for (auto& q : ctx->ring)
        for (auto& ev : q)
            if (ev) cudaEventDestroy(ev);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
    return HJM_OK;
}

hjm_status hjm_ctx_set_stream(hjm_ctx* ctx, void* cuda_stream)
{
    HJM_CHECK_CTX(ctx);
    ctx->stream = cuda_stream ? (cudaStream_t)cuda_stream : ctx->own_stream;
    return HJM_OK;
}

hjm_status hjm_ctx_set_memory_limit(hjm_ctx* ctx, int64_t bytes)
{
    HJM_CHECK_CTX(ctx);
    if (bytes < 0) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "memory limit %lld < 0", (long long)bytes);
    ctx->budget.limit = (size_t)bytes;
    return HJM_OK;
}

hjm_status hjm_ctx_memory_in_use(hjm_ctx* ctx, int64_t* bytes)
{
    HJM_CHECK_CTX(ctx);
    if (!bytes) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "bytes is null");
    *bytes = (int64_t)ctx->budget.used;
    return HJM_OK;
}

hjm_status hjm_ctx_keep_exposures(hjm_ctx* ctx, int32_t keep)
{
    HJM_CHECK_CTX(ctx);
    ctx->keep_exposures = keep != 0;
    return HJM_OK;
}

static bool use_poly_path(const hjm_ctx* ctx) { return ctx->poly_path && ctx->allow_poly_path; }

static bool use_cubic_path(const hjm_ctx* ctx) { return !ctx->poly_path && ctx->cubic_path && ctx->allow_poly_path; }

// 0: table step, 1: quadratic factors, 2: factor k of degree <= k, 3: cubic
// factors with a residual table (FP64 Euler valuations; the other modes run
// the table step on such a market)
static int vol_form_code(const hjm_ctx* ctx)
{
    if (!ctx->have_market) return 0;
    if (use_cubic_path(ctx)) return 3;
    if (!use_poly_path(ctx)) return 0;
    return (ctx->coef[1] == 0.0 && ctx->coef[2] == 0.0 && ctx->coef[5] == 0.0) ? 2 : 1;
}

hjm_status hjm_ctx_set_scheme(hjm_ctx* ctx, int32_t scheme)
{
    HJM_CHECK_CTX(ctx);
    if (scheme != HJM_SCHEME_EULER && scheme != HJM_SCHEME_PREDICTOR_CORRECTOR)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "unknown time scheme %d", scheme);
    ctx->scheme = scheme;
    return HJM_OK;
}

hjm_status hjm_ctx_set_remainder_form(hjm_ctx* ctx, int32_t form)
{
    HJM_CHECK_CTX(ctx);
    if (form != HJM_REMAINDER_AUTO && form != HJM_REMAINDER_CONVECT && form != HJM_REMAINDER_RESPONSE)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "unknown remainder form %d", form);
    ctx->remainder = form;
    return HJM_OK;
}

hjm_status hjm_ctx_remainder_form(hjm_ctx* ctx, int32_t* form)
{
    HJM_CHECK_CTX(ctx);
    if (!form) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "form must not be null");
    *form = ctx->rep_run.remainder;
    return HJM_OK;
}

hjm_status hjm_ctx_set_vol_decomposition(hjm_ctx* ctx, int32_t enable)
{
    HJM_CHECK_CTX(ctx);
    ctx->allow_poly_path = enable != 0;
    return HJM_OK;
}

hjm_status hjm_ctx_vol_decomposition(hjm_ctx* ctx, int32_t* active)
{
    HJM_CHECK_CTX(ctx);
    if (!active) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "active must not be null");
    *active = vol_form_code(ctx);
    return HJM_OK;
}

// ---------------------------------------------------------------------------
// inputs
// ---------------------------------------------------------------------------
// Is every factor row of the volatility table a polynomial of degree <= 2 in
// T = dtau t?  The quadratic through the rows' values at t = 0, mid, last
// (Lagrange form) must reproduce every entry to 1e-12 of the row's largest
// magnitude; its monomial coefficients go to coef[k * 3 + d].
namespace hjm {
// The quadratic fit of a volatility table (factor-major [3][nt]) that decides
// the decomposition: true with coef [3][3] when every factor is a polynomial of
// degree <= 2 to 1e-12 of its scale.  Internal to the library (hjm_run_static
// uses it too).
__attribute__((visibility("hidden"))) bool fit_quadratic_vols(const double* vol, int nt, double dtau, double* coef)
{
    if (nt < 3) return false;
    const int i0 = 0, i1 = (nt - 1) / 2, i2 = nt - 1;
    const double x0 = dtau * i0, x1 = dtau * i1, x2 = dtau * i2;
    for (int k = 0; k < HJM_N_FACTOR; ++k) {
        const double* v = vol + (size_t)k * nt;
        // Lagrange basis l_j(x) = prod (x - x_m) / (x_j - x_m) expanded in 1, x, x^2
        const double d0 = (x0 - x1) * (x0 - x2), d1 = (x1 - x0) * (x1 - x2), d2 = (x2 - x0) * (x2 - x1);
        const double w0 = v[i0] / d0, w1 = v[i1] / d1, w2 = v[i2] / d2;
        double c2 = w0 + w1 + w2;
        double c1 = -(w0 * (x1 + x2) + w1 * (x0 + x2) + w2 * (x0 + x1));
        const double c0 = w0 * x1 * x2 + w1 * x0 * x2 + w2 * x0 * x1;
        double scale = 0.0;
        for (int t = 0; t < nt; ++t) scale = std::max(scale, std::fabs(v[t]));
        // a term below rounding over the whole grid is an exact zero of the
        // factor (lower-degree factors then take the cheaper projection)
        if (std::fabs(c1) * x2 <= 1e-14 * scale) c1 = 0.0;
        if (std::fabs(c2) * x2 * x2 <= 1e-14 * scale) c2 = 0.0;
        for (int t = 0; t < nt; ++t) {
            const double T = dtau * t;
            if (std::fabs(c0 + c1 * T + c2 * T * T - v[t]) > 1e-12 * scale) return false;
        }
        coef[k * 3 + 0] = c0;
        coef[k * 3 + 1] = c1;
        coef[k * 3 + 2] = c2;
    }
    return true;
}

// Cubic factors up to a residual table.  Each factor row is fitted by least
// squares (modified Gram-Schmidt on 1, u, u^2, u^3 with u = (T - T_L) / T_L in
// [-1, 0], then scaled to powers of t = T - T_L) with the lowest degree <= 3
// whose largest residual is at most 2^-20 of the row's largest magnitude;
// coef[k * 4 + d] multiplies t^d, degs[k] is the degree, resid[k * nt + t] =
// sigma_k(T_t) - poly_k(T_t) in FP64.  False when some row needs more than a
// cubic.  A PCA table printed to a fixed number of decimals (the reference's,
// simulation_gpu_testing.cpp:47-63: its factors 2 and 3 are cubics to the
// 9-decimal rounding, 1.1e-7 of their scale) fits with a residual of that
// rounding's size.  Internal to the library.
__attribute__((visibility("hidden"))) bool fit_cubic_resid(const double* vol, int nt, double dtau, double* coef,
                                                            int* degs, double* resid)
{
    if (nt < 5) return false;
    if (nt > HJM_MAX_TENOR) return false;
    const double TL = dtau * (nt - 1);
    const double tol = 0x1p-20;
    double u[HJM_MAX_TENOR], q[4 * HJM_MAX_TENOR], r[HJM_MAX_TENOR];  // no heap use (hjm_run_static calls this)
    for (int t = 0; t < nt; ++t) u[t] = (dtau * t - TL) / TL;
    for (int k = 0; k < HJM_N_FACTOR; ++k) {
        const double* v = vol + (size_t)k * nt;
        double scale = 0.0;
        for (int t = 0; t < nt; ++t) scale = std::max(scale, std::fabs(v[t]));
        bool found = false;
        for (int d = 0; d <= 3 && !found; ++d) {
            // Q R of the columns u^0 .. u^d, then R b = Q^T v
            double R[4][4] = {};
            for (int j = 0; j <= d; ++j) {
                double* qj = &q[(size_t)j * nt];
                for (int t = 0; t < nt; ++t) qj[t] = std::pow(u[t], j);
                for (int i = 0; i < j; ++i) {
                    const double* qi = &q[(size_t)i * nt];
                    double dot = 0.0;
                    for (int t = 0; t < nt; ++t) dot += qi[t] * qj[t];
                    R[i][j] = dot;
                    for (int t = 0; t < nt; ++t) qj[t] -= dot * qi[t];
                }
                double nrm = 0.0;
                for (int t = 0; t < nt; ++t) nrm += qj[t] * qj[t];
                nrm = std::sqrt(nrm);
                R[j][j] = nrm;
                for (int t = 0; t < nt; ++t) qj[t] /= nrm;
            }
            double z[4] = {}, b[4] = {};
            for (int t = 0; t < nt; ++t) r[t] = v[t];
            for (int i = 0; i <= d; ++i) {
                const double* qi = &q[(size_t)i * nt];
                double dot = 0.0;
                for (int t = 0; t < nt; ++t) dot += qi[t] * r[t];
                z[i] = dot;
                for (int t = 0; t < nt; ++t) r[t] -= dot * qi[t];
            }
            for (int i = d; i >= 0; --i) {
                double acc = z[i];
                for (int j = i + 1; j <= d; ++j) acc -= R[i][j] * b[j];
                b[i] = acc / R[i][i];
            }
            double a[4] = {0.0, 0.0, 0.0, 0.0}, sc = 1.0;
            for (int i = 0; i <= d; ++i, sc *= TL) a[i] = b[i] / sc;
            double worst = 0.0;
            for (int t = 0; t < nt; ++t) {
                const double x = dtau * t - TL;
                const double pv = ((a[3] * x + a[2]) * x + a[1]) * x + a[0];
                r[t] = v[t] - pv;
                worst = std::max(worst, std::fabs(r[t]));
            }
            if (worst <= tol * scale) {
                found = true;
                degs[k] = d;
                for (int i = 0; i < 4; ++i) coef[k * 4 + i] = a[i];
                for (int t = 0; t < nt; ++t) resid[(size_t)k * nt + t] = r[t];
            }
        }
        if (!found) return false;
    }
    return true;
}
}  // namespace hjm

static void trapezoid_drift(const std::vector<double>& vol, int nt, double dtau, std::vector<double>& drift)
{
    drift.assign(nt, 0.0);
    for (int k = 0; k < HJM_N_FACTOR; ++k) {
        const double* s = vol.data() + (size_t)k * nt;
        double integral = 0.0;
        for (int i = 0; i < nt; ++i) {
            if (i > 0) integral += 0.5 * (s[i] + s[i - 1]) * dtau;
            drift[i] += s[i] * integral;
        }
    }
}

hjm_status hjm_set_market(hjm_ctx* ctx, int32_t n_tenor, double dtau, const double* spot_host,
                          const double* vol_host, int32_t n_factor, const double* drift_host)
{
    HJM_CHECK_CTX(ctx);
    if (n_tenor < 2 || n_tenor > HJM_MAX_TENOR)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "n_tenor %d outside [2, %d]", n_tenor, HJM_MAX_TENOR);
    if (!path_tenor_supported(n_tenor))
        return fail(ctx, HJM_ERR_UNSUPPORTED, "n_tenor %d: path kernels are built for 51 and 61 tenors", n_tenor);
    if (n_factor != HJM_N_FACTOR)
        return fail(ctx, HJM_ERR_UNSUPPORTED, "n_factor %d: the model has %d factors", n_factor, HJM_N_FACTOR);
    if (!(dtau > 0.0) || !std::isfinite(dtau)) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "dtau must be > 0");
    if (!spot_host || !vol_host) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "spot and vol must not be null");
    if (!finite_all(spot_host, n_tenor) || !finite_all(vol_host, (size_t)n_tenor * n_factor) ||
        (drift_host && !finite_all(drift_host, n_tenor)))
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "market inputs must be finite");
    ctx->nt = n_tenor;
    ctx->dtau = dtau;
    ctx->spot.assign(spot_host, spot_host + n_tenor);
    ctx->vol.assign(vol_host, vol_host + (size_t)n_tenor * n_factor);
    if (drift_host)
        ctx->drift.assign(drift_host, drift_host + n_tenor);
    else
        trapezoid_drift(ctx->vol, n_tenor, dtau, ctx->drift);
    ctx->have_market = true;
    ctx->have_poly = false;
    ctx->poly_path = fit_quadratic_vols(ctx->vol.data(), n_tenor, dtau, ctx->coef);
    ctx->resid.assign((size_t)HJM_N_FACTOR * n_tenor, 0.0);
    ctx->cubic_path = !ctx->poly_path &&
                      fit_cubic_resid(ctx->vol.data(), n_tenor, dtau, &ctx->cubic[0][0], ctx->cubic_degs,
                                      ctx->resid.data());
    if (ctx->have_product && (int)ctx->payA.size() != n_tenor) ctx->have_product = false;
    return HJM_OK;
}

hjm_status hjm_set_market_poly(hjm_ctx* ctx, int32_t n_tenor, double dtau, const double* spot_host,
                               const double* vol_coef_host)
{
    HJM_CHECK_CTX(ctx);
    if (!vol_coef_host) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "vol_coef must not be null");
    if (!finite_all(vol_coef_host, HJM_N_VOL_COEF))
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "volatility coefficients must be finite");
    if (n_tenor < 2 || n_tenor > HJM_MAX_TENOR)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "n_tenor %d outside [2, %d]", n_tenor, HJM_MAX_TENOR);
    std::vector<double> vol((size_t)HJM_N_FACTOR * n_tenor);
    for (int k = 0; k < HJM_N_FACTOR; ++k)
        for (int t = 0; t < n_tenor; ++t) {
            const double T = dtau * t;
            vol[(size_t)k * n_tenor + t] =
                vol_coef_host[k * 3 + 0] + vol_coef_host[k * 3 + 1] * T + vol_coef_host[k * 3 + 2] * T * T;
        }
    hjm_status st = hjm_set_market(ctx, n_tenor, dtau, spot_host, vol.data(), HJM_N_FACTOR, nullptr);
    if (st != HJM_OK) return st;
    std::memcpy(ctx->coef, vol_coef_host, sizeof(ctx->coef));
    ctx->have_poly = true;
    ctx->poly_path = true;
    ctx->cubic_path = false;
    return HJM_OK;
}

hjm_status hjm_set_swap(hjm_ctx* ctx, double notional, double fixed_rate, const double* accrual_host, int32_t payer)
{
    HJM_CHECK_CTX(ctx);
    if (!ctx->have_market) return fail(ctx, HJM_ERR_NOT_CONFIGURED, "hjm_set_market must come first");
    if (!accrual_host) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "accrual must not be null");
    if (!std::isfinite(notional) || !std::isfinite(fixed_rate) || !finite_all(accrual_host, ctx->nt))
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "swap inputs must be finite");
    const double sign = payer ? 1.0 : -1.0;
    ctx->payA.assign(ctx->nt, 0.0);
    ctx->payB.assign(ctx->nt, 0.0);
    for (int i = 0; i < ctx->nt; ++i) {
        ctx->payA[i] = sign * notional * accrual_host[i];
        ctx->payB[i] = sign * notional * accrual_host[i] * fixed_rate;
    }
    ctx->have_product = true;
    return HJM_OK;
}

hjm_status hjm_set_netting_set(hjm_ctx* ctx, int32_t n_swaps, const double* notional_host,
                               const double* fixed_rate_host, const int32_t* n_periods_host,
                               const int32_t* payer_host)
{
    HJM_CHECK_CTX(ctx);
    if (!ctx->have_market) return fail(ctx, HJM_ERR_NOT_CONFIGURED, "hjm_set_market must come first");
    if (n_swaps <= 0 || !notional_host || !fixed_rate_host || !n_periods_host || !payer_host)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "netting set needs n_swaps > 0 and four non-null arrays");
    ctx->payA.assign(ctx->nt, 0.0);
    ctx->payB.assign(ctx->nt, 0.0);
    for (int s = 0; s < n_swaps; ++s) {
        const int np = n_periods_host[s];
        if (np < 1 || np > ctx->nt - 1)
            return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "swap %d: n_periods %d outside [1, %d]", s, np, ctx->nt - 1);
        if (!std::isfinite(notional_host[s]) || !std::isfinite(fixed_rate_host[s]))
            return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "swap %d: non-finite notional or rate", s);
        const double sign = payer_host[s] ? 1.0 : -1.0;
        for (int i = 1; i <= np; ++i) {
            ctx->payA[i] += sign * notional_host[s] * ctx->dtau;
            ctx->payB[i] += sign * notional_host[s] * ctx->dtau * fixed_rate_host[s];
        }
    }
    ctx->have_product = true;
    return HJM_OK;
}

// ---------------------------------------------------------------------------
// valuation
// ---------------------------------------------------------------------------
struct RunShape {
    int stride = 0, B = 0;
};

// Largest growth exponent of the growth-scaled FP32 curve: the scaled noise,
// |phi| <= 5.8 times e^growth, stays below 1e36 (FP32 overflows at 3.4e38).
constexpr double kMaxGrowthFp32 = 80.0;

static hjm_status check_run(hjm_ctx* ctx, int64_t n_paths, int32_t n_steps, double dt, int32_t precision,
                            double hazard, double recovery, double pfe_q, RunShape& sh)
{
    if (!ctx->have_market) return fail(ctx, HJM_ERR_NOT_CONFIGURED, "no market: call hjm_set_market");
    if (!ctx->have_product) return fail(ctx, HJM_ERR_NOT_CONFIGURED, "no product: call hjm_set_swap");
    if (n_paths <= 0 || n_paths > (int64_t)1 << 31)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "n_paths %lld outside [1, 2^31]", (long long)n_paths);
    if (!(dt > 0.0) || !std::isfinite(dt)) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "dt must be > 0");
    if (precision != HJM_PRECISION_FP64 && precision != HJM_PRECISION_MIXED)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "unknown precision %d", precision);
    if (!(hazard >= 0.0) || !std::isfinite(hazard) || !(recovery >= 0.0 && recovery <= 1.0))
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "hazard must be >= 0 and recovery in [0, 1]");
    if (!(pfe_q < 1.0) || std::isnan(pfe_q))
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "pfe_quantile must be < 1 (<= 0 disables PFE)");
    // stride = dtau / dt; the reference truncates (int)(dtau/dt) (simulation_gpu.cu:383);
    // here it must be an integer up to rounding
    const double r = ctx->dtau / dt;
    const long st = std::lround(r);
    if (st < 1 || std::fabs(r - (double)st) > 1e-9 * r)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "dtau/dt = %.17g is not an integer number of steps", r);
    if (st < 2)
        return fail(ctx, HJM_ERR_UNSUPPORTED, "dt must be at most dtau/2 (the kernels need c = dt/dtau < 1)");
    if (n_steps <= 0 || n_steps % st != 0)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "n_steps %d is not a positive multiple of the block length %ld",
                    n_steps, st);
    const int B = n_steps / (int)st;
    if (B > ctx->nt - 1)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT,
                    "%d sampled dates need %d tenors; the grid has %d (n_steps * dt must not exceed the last tenor)",
                    B, B + 1, ctx->nt);
    const size_t smem = ctx->scheme == HJM_SCHEME_PREDICTOR_CORRECTOR
                            ? pc_smem(ctx->nt, B, precision == HJM_PRECISION_MIXED)
                            : path_smem(ctx->nt, B, precision == HJM_PRECISION_MIXED);
    if (smem > 227 * 1024) return fail(ctx, HJM_ERR_UNSUPPORTED, "shared memory %zu B exceeds 227 KB", smem);
    // the growth-scaled curve grows by (1 + rr)^n_steps, rr = c / (1 - c); in
    // FP32 the scaled noise must stay far from overflow
    const double cc = dt / ctx->dtau;
    const double growth = (double)n_steps * std::log1p(cc / (1.0 - cc));
    if (precision == HJM_PRECISION_MIXED && growth > kMaxGrowthFp32)
        return fail(ctx, HJM_ERR_UNSUPPORTED,
                    "mixed precision: %d steps at dt/dtau = %.6g grow the scaled curve by e^%.1f (limit e^%.0f); "
                    "use FP64 or a smaller dt",
                    n_steps, cc, growth, kMaxGrowthFp32);
    sh.stride = (int)st;
    sh.B = B;
    return HJM_OK;
}

// Deterministic curve p (no noise) in FP64: p_n = spot for the first block,
// then p_{n+1}[t] = p_n[t] + (mu[t] dt + (dF/dtau) dt) (simulation_cpu.h:37-54
// with zero normals); its samples and discount integrals per tenor.
static void deterministic_curve(const hjm_ctx* ctx, int stride, int B, double dt, double* psamp, double* psum)
{
    const int nt = ctx->nt;
    std::vector<double> p(ctx->spot), pn(nt), acc(nt, 0.0), ps(nt);
    // drift term a(f)[t] = mu[t] + dF/dtau (forward difference, backward at the last tenor)
    auto drift_term = [&](const std::vector<double>& f, int t) {
        const double dF = (t == nt - 1) ? f[t] - f[t - 1] : f[t + 1] - f[t];
        return ctx->drift[t] + dF / ctx->dtau;
    };
    for (int i = 0; i < kMaxTenor; ++i) psamp[i] = psum[i] = 0.0;
    for (int s = 0; s < stride; ++s)
        for (int t = 0; t < nt; ++t) acc[t] += p[t];
    psamp[1] = p[1];
    psum[1] = acc[1];
    for (int b = 1; b < B; ++b) {
        for (int s = 0; s < stride; ++s) {
            if (ctx->scheme == HJM_SCHEME_PREDICTOR_CORRECTOR) {
                for (int t = 0; t < nt; ++t) ps[t] = p[t] + drift_term(p, t) * dt;
                for (int t = 0; t < nt; ++t) pn[t] = p[t] + 0.5 * (drift_term(p, t) + drift_term(ps, t)) * dt;
            } else {
                for (int t = 0; t < nt; ++t) {
                    const double dF = (t == nt - 1) ? p[t] - p[t - 1] : p[t + 1] - p[t];
                    double dfbar = ctx->drift[t] * dt;
                    dfbar += (dF / ctx->dtau) * dt;
                    pn[t] = p[t] + dfbar;
                }
            }
            for (int t = 0; t < nt; ++t) {
                p[t] = pn[t];
                acc[t] += p[t];
            }
        }
        psamp[b + 1] = p[b + 1];
        psum[b + 1] = acc[b + 1];
    }
}


template <typename T>
static void fill_params(const hjm_ctx* ctx, const RunShape& sh, int64_t n_paths, double dt, uint64_t seed,
                        uint64_t path_offset, double hazard, double recovery, int64_t ld, bool store,
                        PathParams<T>& P, FinalParams& F)
{
    std::memset(&P, 0, sizeof(P));
    std::memset(&F, 0, sizeof(F));
    const int nt = ctx->nt;
    const double sq = std::sqrt(dt);
    for (int k = 0; k < kFactors; ++k)
        for (int t = 0; t < nt; ++t) P.sv[k][t] = (T)(sq * ctx->vol[(size_t)k * nt + t]);
    deterministic_curve(ctx, sh.stride, sh.B, dt, P.psamp, P.psum);
    for (int i = 0; i < nt; ++i) {
        P.payA[i] = ctx->payA[i];
        P.payB[i] = ctx->payB[i];
    }
    for (int j = 1; j <= sh.B; ++j) {
        const double t0 = (j - 1) * ctx->dtau, t1 = j * ctx->dtau;
        const double e0 = std::exp(-hazard * t0), e1 = std::exp(-hazard * t1);
        P.cvaw[j] = (1.0 - recovery) * (e0 - e1);
        F.cvaw[j] = P.cvaw[j];
        F.dcvaw[j] = (1.0 - recovery) * (-t0 * e0 + t1 * e1);
    }
    if (use_poly_path(ctx))
        for (int k = 0; k < kFactors; ++k)
            for (int d = 0; d < 3; ++d) P.svc[k][d] = sq * ctx->coef[k * 3 + d];
    P.k1 = (dt / ctx->dtau) * ctx->dtau;
    P.k2 = (dt / ctx->dtau) * ctx->dtau * ctx->dtau;
    fill_growth_scale(P, dt / ctx->dtau, P.k2, sh.stride, sh.B);
    for (int t = 0; t < nt; ++t) P.tau[t] = (T)(ctx->dtau * t);
    P.c = (T)(dt / ctx->dtau);
    P.dt = dt;
    P.m = 1.0 / ctx->dtau;
    P.inv_m = ctx->dtau;
    P.key0 = (uint32_t)seed;
    P.key1 = (uint32_t)(seed >> 32);
    philox_round_keys(P.key0, P.key1, P.rk0, P.rk1);
    P.inv_c = ctx->dtau / dt;
    P.path_offset = path_offset;
    P.n_paths = n_paths;
    P.ld = ld;
    P.n_blocks = sh.B;
    P.stride = sh.stride;
    P.store_exposures = store ? 1 : 0;
    F.n_paths = n_paths;
    F.n_blocks = sh.B;
}

// Predictor-corrector parameters from the Euler ones: loadings N sqrt(dt)
// sigma (N = I + c Dl / 2), the stencil r1 = a1/a0, r2 = a2/a0 rounded once,
// growth scales and effective coefficients derived from them.
template <typename T>
static void fill_pc(const hjm_ctx* ctx, const RunShape& sh, double dt, const PathParams<T>& P, PcParams<T>& Q)
{
    std::memset(&Q, 0, sizeof(Q));
    Q.P = P;
    const int nt = ctx->nt;
    const double c = dt / ctx->dtau, sq = std::sqrt(dt);
    for (int k = 0; k < kFactors; ++k) {
        const double* sig = ctx->vol.data() + (size_t)k * nt;
        for (int t = 0; t < nt; ++t) {
            const double d = (t == nt - 1) ? sig[t] - sig[t - 1] : sig[t + 1] - sig[t];
            Q.P.sv[k][t] = (T)(sq * (sig[t] + 0.5 * c * d));
        }
    }
    const double a0 = 1.0 - c + 0.5 * c * c, a1 = c - c * c, a2 = 0.5 * c * c;
    const T r1 = (T)(a1 / a0), r2 = (T)(a2 / a0);
    const double base = 1.0 + (double)r1 + (double)r2;
    for (int b = 0; b < kMaxTenor; ++b) {
        const double e = (b >= 1 && b <= sh.B) ? (double)((b - 1) * sh.stride) : 0.0;
        Q.P.gblk[b] = (T)std::pow(base, -e);
        Q.P.igblk[b] = (T)std::pow(base, e);
    }
    Q.P.ip = (T)base;
    Q.r1 = r1;
    Q.r2 = r2;
    const double ce = ((double)r1 + 2.0 * (double)r2) / base;
    Q.a0e = (T)(1.0 / base);
    Q.a1e = (T)((double)r1 / base);
    Q.a2e = (T)((double)r2 / base);
    Q.ce = (T)ce;
    Q.inv_1ma0 = (T)(base / ((double)r1 + (double)r2));
    Q.inv_ce = (T)(1.0 / ce);
    // polynomial form: N xi = (alpha + c dtau beta / 2 + c dtau^2 gamma / 2) + (beta + c dtau gamma) T
    // + gamma T^2 - c dtau^2 gamma e_L;  A2 T^2 = T^2 + 2 c dtau T + (c + c^2) dtau^2
    // - c^2 dtau^2 e_{L-1} - (2c + c^2) dtau^2 e_L
    const double dtau = ctx->dtau;
    for (int k = 0; k < kFactors; ++k) {
        const double c0 = sq * ctx->coef[3 * k], c1 = sq * ctx->coef[3 * k + 1], c2 = sq * ctx->coef[3 * k + 2];
        Q.aS[k] = (T)(c0 + 0.5 * c * dtau * c1 + 0.5 * c * dtau * dtau * c2);
        Q.aU[k] = (T)(c1 + c * dtau * c2);
        Q.aW[k] = (T)c2;
    }
    Q.k1 = (T)(c * dtau);
    Q.k2p = (T)((c + c * c) * dtau * dtau);
    Q.k1x2 = (T)(2.0 * c * dtau);
    Q.wL1 = (T)(-c * c * dtau * dtau);
    Q.wL = (T)(-(2.0 * c + c * c) * dtau * dtau);
    Q.gL = (T)(-c * dtau * dtau);
}

// FP64 valuation with a decomposition (quadratic factors under either
// scheme, or cubic ones with a residual table under the Euler step): the
// response form of hjm_eresp.cu, whose per-step work is on the FP32 pipe and
// which takes any number of dates (in windows); measured 9.0x the convected
// form at 20 dates (Euler), and the convected cubic has no form but the table
// step, so AUTO always takes it.
//
// Volatility-table step (no decomposition): the whole stochastic curve in
// impulse responses, per step and date still to be sampled three
// double-FP32 terms on the FP32 pipe (in windows of 16 dates), against four
// FP64 FMAs per live tenor (five for the predictor-corrector) when convected.
//
// Mixed precision with polynomial factors (either scheme) and the adjoint
// without checkpoints (Euler): the FP32 response form of hjm_mresp.cu when
// the dates whose responses count fit its slots (mresp_slots: the 10y swap's
// 20 dates in 8), else the convected pairs.
static bool use_response_form(const hjm_ctx* ctx) { return ctx->remainder != HJM_REMAINDER_CONVECT; }

// The volatility-table response table of the run shape, scheme and loadings
// sv [kFactors][kMaxTenor] (the path parameters'), on the stream: rebuilt
// only when it changed, after the kernels of earlier valuations that read it.
static hjm_status ensure_vol_response_table(hjm_ctx* ctx, const RunShape& sh, double dt, const double* sv,
                                            cudaStream_t s)
{
    const double c = dt / ctx->dtau;
    const int nt = ctx->nt;
    std::vector<double> key((size_t)kFactors * nt);
    for (int k = 0; k < kFactors; ++k)
        for (int t = 0; t < nt; ++t) key[(size_t)k * nt + t] = sv[k * kMaxTenor + t];
    hjm_ctx::VrespKey& k = ctx->vresp_key;
    if (!ctx->resp_used) HJM_CUDA(ctx, cudaEventCreateWithFlags(&ctx->resp_used, cudaEventDisableTiming));
    if (k.valid && k.nt == nt && k.stride == sh.stride && k.B == sh.B && k.c == c && k.scheme == ctx->scheme &&
        k.sv == key)
        return HJM_OK;
    k.valid = false;
    const size_t bytes = sizeof(float4) * response_table_vol_elems(sh.stride, sh.B);
    if (bytes > ctx->vresp.bytes)
        HJM_CUDA(ctx, ctx->vresp.ensure(bytes));  // cudaFree waits for the device
    else
        HJM_CUDA(ctx, cudaStreamWaitEvent(s, ctx->resp_used, 0));
    HJM_CUDA(ctx, cudaMemsetAsync(ctx->vresp.p, 0, bytes, s));  // entries the kernel reads as exact zeros
    HJM_CUDA(ctx, launch_response_table_vol(nt, c, sh.stride, sh.B, ctx->scheme == HJM_SCHEME_PREDICTOR_CORRECTOR, sv,
                                            (float4*)ctx->vresp.p, s));
    ctx->stat_launches += 1;
    k.nt = nt;
    k.stride = sh.stride;
    k.B = sh.B;
    k.c = c;
    k.scheme = ctx->scheme;
    k.sv = key;
    k.valid = true;
    return HJM_OK;
}

// The response form's table (remainder and residual responses, frame
// coefficients, active prefixes) for the run shape and decomposition, on the
// stream: rebuilt only when they changed, after the kernels of earlier
// valuations that read it.
static hjm_status ensure_eresp_table(hjm_ctx* ctx, const RunShape& sh, double dt,
                                     const std::vector<EulerRespFrame>& frames, const std::vector<double>& resid,
                                     int nres, bool pc, cudaStream_t s)
{
    const EulerRespFrame& fr = frames[0];
    const double c = dt / ctx->dtau;
    hjm_ctx::ErespKey& k = ctx->eresp_key;
    if (!ctx->resp_used) HJM_CUDA(ctx, cudaEventCreateWithFlags(&ctx->resp_used, cudaEventDisableTiming));
    if (k.valid && k.pc == pc && k.nt == ctx->nt && k.stride == sh.stride && k.B == sh.B && k.np == fr.np && k.c == c &&
        k.dtau == ctx->dtau && k.nres == nres && k.frames.size() == frames.size() &&
        std::memcmp(k.frames.data(), frames.data(), sizeof(EulerRespFrame) * frames.size()) == 0 && k.resid == resid)
        return HJM_OK;
    k.valid = false;
    const size_t bytes = sizeof(float4) * eresp_table_elems(sh.stride, sh.B, fr.np, nres, (int)frames.size());
    if (bytes > ctx->eresp.bytes)
        HJM_CUDA(ctx, ctx->eresp.ensure(bytes));  // cudaFree waits for the device
    else
        HJM_CUDA(ctx, cudaStreamWaitEvent(s, ctx->resp_used, 0));
    HJM_CUDA(ctx, launch_eresp_tables(ctx->nt, c, ctx->dtau, sh.stride, sh.B, frames.data(), (int)frames.size(),
                                      resid.empty() ? nullptr : resid.data(), nres, pc, (float4*)ctx->eresp.p, s));
    ctx->stat_launches += 3;
    k.pc = pc;
    k.nt = ctx->nt;
    k.stride = sh.stride;
    k.B = sh.B;
    k.np = fr.np;
    k.nres = nres;
    k.c = c;
    k.dtau = ctx->dtau;
    k.frames = frames;
    k.resid = resid;
    k.valid = true;
    return HJM_OK;
}

// An FP64 valuation in the response form (hjm_eresp.cu): the parts' frame
// and loadings of the market's decomposition, the table, the carry of a
// windowed run, and one launch per window.  Q: the predictor-corrector's
// parameters (its parts' step, N-projected loadings and deterministic
// curve; quadratic factors), or null for the Euler step.
static hjm_status enqueue_eresp(hjm_ctx* ctx, const RunShape& sh, double dt, const PathParams<double>& P,
                                const double* ext_dev, double* estore, cudaStream_t s,
                                const PcParams<double>* Q = nullptr)
{
    const bool pc = Q != nullptr;
    const bool cubic = !pc && use_cubic_path(ctx);
    std::vector<double> resid;
    int nres = 0;
    if (cubic) {
        const double sq = std::sqrt(dt);
        resid.resize(ctx->resid.size());
        for (size_t i = 0; i < resid.size(); ++i) resid[i] = sq * ctx->resid[i];
        nres = eresp_residual_factors(ctx->resid.data(), ctx->vol.data(), ctx->nt);
    }
    // the earliest date the remainder reaches (the windows hold slots from it on)
    const double c = dt / ctx->dtau;
    hjm_ctx::ErespFirst& fa = ctx->eresp_first;
    if (!(fa.valid && fa.pc == pc && fa.nt == ctx->nt && fa.stride == sh.stride && fa.B == sh.B && fa.nres == nres &&
          fa.c == c)) {
        fa.first = eresp_first_active_date(ctx->nt, c, sh.stride, sh.B, nres, pc);
        fa.pc = pc;
        fa.nt = ctx->nt;
        fa.stride = sh.stride;
        fa.B = sh.B;
        fa.nres = nres;
        fa.c = c;
        fa.valid = true;
    }
    int lo[kMaxTenor], hi[kMaxTenor];
    const int n_windows = eresp_windows(sh.B, fa.first, lo, hi, nullptr, eresp_window_dates(nres));
    std::vector<EulerRespFrame> frames(n_windows);
    int degs = 0;
    double svc_pc[kFactors][3];  // the predictor-corrector's N-projected loadings of 1, T, T^2
    if (pc)
        for (int k = 0; k < kFactors; ++k) {
            svc_pc[k][0] = Q->aS[k];
            svc_pc[k][1] = Q->aU[k];
            svc_pc[k][2] = Q->aW[k];
        }
    for (int w = 0; w < n_windows; ++w)
        eresp_make_frame(dt, ctx->dtau, ctx->nt, pc ? svc_pc : P.svc, cubic ? &ctx->cubic[0][0] : nullptr,
                         ctx->cubic_degs, eresp_window_centre(ctx->dtau, lo[w], hi[w]), frames[w], degs, pc);
    const EulerRespFrame& fr = frames[0];
    const size_t smem = eresp_max_smem(sh.B, fr.np, sh.stride, fa.first, nres);
    if (smem > 227 * 1024) return fail(ctx, HJM_ERR_UNSUPPORTED, "shared memory %zu B exceeds 227 KB", smem);
    hjm_status st = ensure_eresp_table(ctx, sh, dt, frames, resid, nres, pc, s);
    if (st != HJM_OK) return st;
    EulerRespParams E;
    std::memset(&E, 0, sizeof(E));
    E.P = P;
    E.wnew_L = pc ? Q->gL : 0.0;
    E.tenor_L = ctx->nt - 1;
    E.frame = block_frame_n(fr.n, sh.stride);
    E.row = eresp_row(sh.B);
    // the pairs are renormalised for the residual's terms and for runs of more
    // than 25 dates, whose dates near the last tenor carry large remainders
    E.renorm = (cubic || sh.B > kRespSlots + 1) ? 1 : 0;
    double* carry = nullptr;
    if (n_windows > 1) {
        HJM_CUDA(ctx, ctx->carry.ensure(sizeof(double) * 2 * (size_t)P.n_paths));
        carry = (double*)ctx->carry.p;
    }
    int launches = 0;
    HJM_CUDA(ctx, launch_path_fp64_eresp(E, frames.data(), degs, nres, (const float4*)ctx->eresp.p, fa.first, ext_dev,
                                         (double*)ctx->partials.p, estore, carry, s, &launches));
    ctx->stat_launches += launches - 1;
    return HJM_OK;
}

// Mixed precision on a market whose factors are cubics up to a residual
// (hjm_set_market's fit): the cubic polynomial form of the mixed kernel, in
// powers of t = T - tau0 about the middle of the sampled tenors (the cubic's
// terms cancel least there), the fit re-expanded on the host in FP64 and
// rounded to FP32.  The residual, at most 2^-20 of each factor's scale by the
// fit's rule (1.1e-7 for the reference driver's PCA table: two FP32 ulps of
// the loadings, which the table step rounds to half an ulp), is left out: an
// input perturbation of that size, far inside the mixed precision's 1e-4.
namespace hjm {
// (Shared with hjm_run_static; internal to the library.)  cubic: [3][4]
// coefficients of (T - T_L)^d as fit_cubic_resid gives them.
__attribute__((visibility("hidden"))) void mixed_cubic_params(int nt, double dtau, double dt, int n_blocks,
                                                              const double* cubic, MixedParams& M)
{
    const double c = dt / dtau, sq = std::sqrt(dt);
    const double TL = dtau * (nt - 1);
    const double tau0 = eresp_window_centre(dtau, 1, n_blocks);
    const double dl = tau0 - TL;  // sum_e a_e (T - T_L)^e = sum_d a'_d (T - tau0)^d
    for (int k = 0; k < kFactors; ++k) {
        const double* a = cubic + 4 * k;
        const double sh4[4] = {a[0] + dl * (a[1] + dl * (a[2] + dl * a[3])), a[1] + dl * (2.0 * a[2] + 3.0 * dl * a[3]),
                               a[2] + 3.0 * dl * a[3], a[3]};
        for (int d = 0; d < 3; ++d) M.svcf[k][d] = (float)(sq * sh4[d]);
        M.svcx[k] = (float)(sq * sh4[3]);
    }
    M.k3f = (float)(c * dtau * dtau * dtau);
    M.src3f = (float)(3.0 * (TL - tau0));
    for (int t = 0; t < nt; ++t) M.P.tau[t] = (float)(dtau * t - tau0);
}
}  // namespace hjm

// The date slots of the mixed-precision response form for the run shape and
// scheme (0: the run convects), counted on the host once per shape.
static int mresp_run_slots(hjm_ctx* ctx, const RunShape& sh, double dt, bool pc = false)
{
    const double c = dt / ctx->dtau;
    hjm_ctx::MrespKey& k = ctx->mresp_key;
    if (!(k.valid && k.pc == pc && k.nt == ctx->nt && k.stride == sh.stride && k.B == sh.B && k.c == c &&
          k.dtau == ctx->dtau)) {
        k.ns = mresp_slots(ctx->nt, c, ctx->dtau, sh.stride, sh.B, pc);
        k.pc = pc;
        k.nt = ctx->nt;
        k.stride = sh.stride;
        k.B = sh.B;
        k.c = c;
        k.dtau = ctx->dtau;
        k.valid = true;
        k.on_device = false;
    }
    return k.ns;
}

// Its table on the stream (for the shape mresp_run_slots counted): built
// only when the shape changed, after the kernels of earlier valuations that
// read the old one.
static hjm_status ensure_mresp_table(hjm_ctx* ctx, cudaStream_t s)
{
    hjm_ctx::MrespKey& k = ctx->mresp_key;
    if (k.on_device) return HJM_OK;
    if (!ctx->resp_used) HJM_CUDA(ctx, cudaEventCreateWithFlags(&ctx->resp_used, cudaEventDisableTiming));
    const size_t bytes = sizeof(float4) * mresp_table_elems(k.stride, k.B, k.ns);
    if (bytes > ctx->mresp.bytes)
        HJM_CUDA(ctx, ctx->mresp.ensure(bytes));  // cudaFree waits for the device
    else
        HJM_CUDA(ctx, cudaStreamWaitEvent(s, ctx->resp_used, 0));
    HJM_CUDA(ctx, launch_mresp_table(k.nt, k.c, k.dtau, k.stride, k.B, k.ns, k.pc, (float4*)ctx->mresp.p, s));
    ctx->stat_launches += 1;
    k.on_device = true;
    return HJM_OK;
}

// The volatility-table step in the response form (its table already on the
// stream): the carry of a windowed run, one launch per window.
static hjm_status enqueue_vresp(hjm_ctx* ctx, const RunShape& sh, const PathParams<double>& P, const double* ext_dev,
                                double* estore, cudaStream_t s)
{
    double* carry = nullptr;
    if (vresp_windows(sh.B) > 1) {
        HJM_CUDA(ctx, ctx->carry.ensure(sizeof(double) * 2 * (size_t)P.n_paths));
        carry = (double*)ctx->carry.p;
    }
    int launches = 0;
    HJM_CUDA(ctx, launch_path_fp64_vresp(ctx->nt, P, (const float4*)ctx->vresp.p, ext_dev, (double*)ctx->partials.p,
                                         estore, carry, s, &launches));
    ctx->stat_launches += launches - 1;
    return HJM_OK;
}

static hjm_status enqueue_impl(hjm_ctx* ctx, int64_t n_paths, int32_t n_steps, double dt, uint64_t seed,
                               uint64_t path_offset, int32_t precision, double hazard, double recovery, double pfe_q,
                               const double* ext_dev)
{
    RunShape sh;
    hjm_status st = check_run(ctx, n_paths, n_steps, dt, precision, hazard, recovery, pfe_q, sh);
    if (st != HJM_OK) return st;
    HJM_CUDA(ctx, cudaSetDevice(ctx->device));
    const bool mixed = precision == HJM_PRECISION_MIXED;
    const bool want_pfe = pfe_q > 0.0;
    const bool store = want_pfe || ctx->keep_exposures;
    const int n_dates = sh.B + 1;
    const int R = sh.B + 3;
    const bool pc = ctx->scheme == HJM_SCHEME_PREDICTOR_CORRECTOR;
    // a cubic market in mixed precision (Euler): the cubic polynomial form
    const bool mixed_cubic = mixed && !pc && use_cubic_path(ctx);
    // mixed precision with polynomial factors: the response form when the
    // dates its remainder reaches fit its slots (else the convected pairs)
    const int mresp_ns = (mixed && (pc ? use_poly_path(ctx) : (use_poly_path(ctx) || mixed_cubic)) &&
                          use_response_form(ctx))
                             ? mresp_run_slots(ctx, sh, dt, pc)
                             : 0;
    const int cta = mresp_ns ? kCta
                             : (pc ? pc_cta() : path_cta(mixed, ctx->nt, sh.B, use_poly_path(ctx) || mixed_cubic));
    const int64_t n_ctas = (n_paths + cta - 1) / cta;
    const int64_t ld = (n_paths + 3) / 4 * 4;
    const size_t esize = mixed ? 4 : 8;

    HJM_CUDA(ctx, ctx->partials.ensure(sizeof(double) * (size_t)n_ctas * R));
    HJM_CUDA(ctx, ctx->sums.ensure(sizeof(double) * kMaxTenor * 4));
    HJM_CUDA(ctx, ctx->result.ensure(sizeof(double) * kResLen));
    if (store) HJM_CUDA(ctx, ctx->estore.ensure(esize * (size_t)n_dates * (size_t)ld));
    if (want_pfe) {
        HJM_CUDA(ctx, ctx->sel.ensure(sizeof(SelState) * kMaxTenor));
        HJM_CUDA(ctx, ctx->hist.ensure(pfe_scratch_bytes()));
    }
    cudaStream_t s = ctx->stream;
    ctx->have_result = false;
    HJM_CUDA(ctx, cudaMemsetAsync(ctx->result.p, 0, sizeof(double) * kResLen, s));

    FinalParams F;
    ctx->ev = ctx->ring[ctx->n_enqueued % hjm_ctx::kRing];
    ctx->n_enqueued++;
    ctx->stat_launches = 3;  // path kernel, column reduction, finalisation
    ctx->stat_h2d = (mixed ? sizeof(MixedParams) : sizeof(PathParams<double>)) + sizeof(FinalParams);
    ctx->stat_d2h = 0;
    HJM_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
    bool resp = false;
    // the volatility form this run takes (vol_form_code's values): a cubic
    // market runs its decomposition in the Euler step only (FP64: the response
    // form with the residual; mixed precision: the cubic polynomial form)
    int run_form = use_poly_path(ctx) ? vol_form_code(ctx) : 0;
    if (pc && mixed) {
        PathParams<float> P;
        fill_params<float>(ctx, sh, n_paths, dt, seed, path_offset, hazard, recovery, ld, store, P, F);
        PcParams<float> Q;
        fill_pc<float>(ctx, sh, dt, P, Q);
        ctx->stat_h2d = sizeof(Q) + sizeof(FinalParams);
        if (mresp_ns) {
            // the response form: the two-stage step's parts are the Euler
            // kernel's update with the N-projected loadings and (c + c^2) dtau^2
            MixedParams M;
            std::memset(&M, 0, sizeof(M));
            M.P = Q.P;
            for (int k = 0; k < kFactors; ++k) {
                M.svcf[k][0] = Q.aS[k];
                M.svcf[k][1] = Q.aU[k];
                M.svcf[k][2] = Q.aW[k];
            }
            M.k1f = Q.k1;
            M.k2f = Q.k2p;
            st = ensure_mresp_table(ctx, s);
            if (st != HJM_OK) return st;
            HJM_CUDA(ctx, launch_path_mixed_resp(M, mresp_ns, false, (const float4*)ctx->mresp.p, ext_dev,
                                                 (double*)ctx->partials.p, store ? (float*)ctx->estore.p : nullptr,
                                                 s));
            HJM_CUDA(ctx, cudaEventRecord(ctx->resp_used, s));
            resp = true;
        } else {
            HJM_CUDA(ctx, launch_path_pc(ctx->nt, Q, use_poly_path(ctx), ext_dev, (double*)ctx->partials.p,
                                         store ? (float*)ctx->estore.p : nullptr, s));
        }
    } else if (pc) {
        PathParams<double> P;
        fill_params<double>(ctx, sh, n_paths, dt, seed, path_offset, hazard, recovery, ld, store, P, F);
        PcParams<double> Q;
        fill_pc<double>(ctx, sh, dt, P, Q);
        ctx->stat_h2d = sizeof(Q) + sizeof(FinalParams);
        resp = use_response_form(ctx);
        if (resp && use_poly_path(ctx)) {
            // the decomposition in the response form of hjm_eresp.cu, with the
            // two-stage step's parts frame and remainder table (any number of dates)
            st = enqueue_eresp(ctx, sh, dt, Q.P, ext_dev, store ? (double*)ctx->estore.p : nullptr, s, &Q);
            if (st != HJM_OK) return st;
        } else if (resp) {
            st = ensure_vol_response_table(ctx, sh, dt, &Q.P.sv[0][0], s);
            if (st != HJM_OK) return st;
            st = enqueue_vresp(ctx, sh, Q.P, ext_dev, store ? (double*)ctx->estore.p : nullptr, s);
            if (st != HJM_OK) return st;
        } else {
            HJM_CUDA(ctx, launch_path_pc(ctx->nt, Q, use_poly_path(ctx), ext_dev, (double*)ctx->partials.p,
                                         store ? (double*)ctx->estore.p : nullptr, s));
        }
        if (resp) HJM_CUDA(ctx, cudaEventRecord(ctx->resp_used, s));
    } else if (mixed) {
        PathParams<float> P;
        fill_params<float>(ctx, sh, n_paths, dt, seed, path_offset, hazard, recovery, ld, store, P, F);
        MixedParams M;
        pack_mixed_params(ctx->nt, P, M);
        if (mixed_cubic) {
            mixed_cubic_params(ctx->nt, ctx->dtau, dt, sh.B, &ctx->cubic[0][0], M);
            run_form = vol_form_code(ctx);
        }
        if (mresp_ns) {
            st = ensure_mresp_table(ctx, s);
            if (st != HJM_OK) return st;
            HJM_CUDA(ctx, launch_path_mixed_resp(M, mresp_ns, mixed_cubic, (const float4*)ctx->mresp.p, ext_dev,
                                                 (double*)ctx->partials.p, store ? (float*)ctx->estore.p : nullptr,
                                                 s));
            HJM_CUDA(ctx, cudaEventRecord(ctx->resp_used, s));
            resp = true;
        } else {
            HJM_CUDA(ctx, launch_path_mixed(ctx->nt, M, use_poly_path(ctx), ext_dev, (double*)ctx->partials.p,
                                            store ? (float*)ctx->estore.p : nullptr, s, mixed_cubic));
        }
    } else {
        PathParams<double> P;
        fill_params<double>(ctx, sh, n_paths, dt, seed, path_offset, hazard, recovery, ld, store, P, F);
        resp = use_response_form(ctx);
        if (resp && (use_poly_path(ctx) || use_cubic_path(ctx))) {
            st = enqueue_eresp(ctx, sh, dt, P, ext_dev, store ? (double*)ctx->estore.p : nullptr, s);
            if (st != HJM_OK) return st;
            run_form = vol_form_code(ctx);
        } else if (resp) {
            st = ensure_vol_response_table(ctx, sh, dt, &P.sv[0][0], s);
            if (st != HJM_OK) return st;
            st = enqueue_vresp(ctx, sh, P, ext_dev, store ? (double*)ctx->estore.p : nullptr, s);
            if (st != HJM_OK) return st;
        } else {
            // convected: the quadratic decomposition, else the table step
            HJM_CUDA(ctx, launch_path_fp64(ctx->nt, P, use_poly_path(ctx), ext_dev,
                                           (double*)ctx->partials.p, store ? (double*)ctx->estore.p : nullptr, s));
        }
        if (resp) HJM_CUDA(ctx, cudaEventRecord(ctx->resp_used, s));
    }
    HJM_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
    HJM_CUDA(ctx, launch_reduce((const double*)ctx->partials.p, n_ctas, R, (double*)ctx->sums.p, F,
                                (double*)ctx->result.p, s));
    HJM_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
    if (want_pfe) {
        const int64_t k = std::min<int64_t>(std::max<int64_t>((int64_t)std::ceil(pfe_q * (double)n_paths - 1e-7), 1),
                                            n_paths);
        HJM_CUDA(ctx, launch_pfe(ctx->estore.p, !mixed, ld, n_paths, n_dates, (uint64_t)(k - 1),
                                 (SelState*)ctx->sel.p, ctx->hist.p, (double*)ctx->result.p, ctx->n_sms,
                                 s));
        // init, write, per 11-bit digit a histogram and a scan, and between
        // digits the compaction and ranking (6 digits of FP64 keys, 3 of FP32)
        ctx->stat_launches += 2 + (mixed ? 3 * 2 + 2 * 2 : 6 * 2 + 5 * 2);
    }
    HJM_CUDA(ctx, cudaEventRecord(ctx->ev[3], s));
    {
        hjm_ctx::Report& r = ctx->rep_run;
        r = hjm_ctx::Report();
        r.n_paths = n_paths;
        r.n_steps = n_steps;
        r.n_dates = n_dates;
        r.nt = ctx->nt;
        r.precision = precision;
        r.vol_form = run_form;
        r.dt = dt;
        r.dtau = ctx->dtau;
        r.hazard = hazard;
        r.recovery = recovery;
        r.pfe_q = pfe_q;
        r.pfe = want_pfe;
        r.seed = seed;
        r.path_offset = path_offset;
        r.external_normals = ext_dev != nullptr;
        r.scheme = ctx->scheme;
        r.remainder = resp ? 2 : 1;
    }
    ctx->last_n_paths = n_paths;
    ctx->last_n_dates = n_dates;
    ctx->last_mixed = mixed;
    ctx->last_stored = store;
    ctx->last_pfe = want_pfe;
    ctx->last_ld = ld;
    ctx->have_result = true;
    return HJM_OK;
}

hjm_status hjm_enqueue(hjm_ctx* ctx, int64_t n_paths, int32_t n_steps, double dt, uint64_t seed,
                       uint64_t path_offset, int32_t precision, double hazard_rate, double recovery,
                       double pfe_quantile)
{
    HJM_CHECK_CTX(ctx);
    return enqueue_impl(ctx, n_paths, n_steps, dt, seed, path_offset, precision, hazard_rate, recovery, pfe_quantile,
                        nullptr);
}

hjm_status hjm_fetch_results(hjm_ctx* ctx, double* ee_out, double* pfe_out, double* cva_out)
{
    HJM_CHECK_CTX(ctx);
    if (!ctx->have_result) return fail(ctx, HJM_ERR_NOT_CONFIGURED, "no valuation has been enqueued");
    double res[kResLen];
    HJM_CUDA(ctx, cudaSetDevice(ctx->device));
    HJM_CUDA(ctx, cudaMemcpyAsync(res, ctx->result.p, sizeof(res), cudaMemcpyDeviceToHost, ctx->stream));
    HJM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    ctx->stat_d2h += (int64_t)sizeof(res);
    if (ee_out)
        for (int j = 0; j < ctx->nt; ++j) ee_out[j] = res[kResEE + j];
    if (pfe_out)
        for (int j = 0; j < ctx->nt; ++j) pfe_out[j] = ctx->last_pfe ? res[kResPFE + j] : 0.0;
    if (cva_out) {
        cva_out[HJM_CVA_VALUE] = res[kResCVA];
        cva_out[HJM_CVA_STDERR] = res[kResCVAStderr];
        cva_out[HJM_CVA_DHAZARD] = res[kResDCVADHazard];
    }
    hjm_ctx::Report& r = ctx->rep;
    r = ctx->rep_run;
    r.valid = true;
    r.ee.assign(res + kResEE, res + kResEE + ctx->nt);
    if (ctx->last_pfe) r.pfe_v.assign(res + kResPFE, res + kResPFE + ctx->nt);
    r.cva = res[kResCVA];
    r.cva_stderr = res[kResCVAStderr];
    r.dhazard = res[kResDCVADHazard];
    return HJM_OK;
}

hjm_status hjm_run(hjm_ctx* ctx, int64_t n_paths, int32_t n_steps, double dt, uint64_t seed, uint64_t path_offset,
                   int32_t precision, double hazard_rate, double recovery, double pfe_quantile, double* ee_out,
                   double* pfe_out, double* cva_out)
{
    HJM_CHECK_CTX(ctx);
    if (!ee_out && !pfe_out && !cva_out) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "no output requested");
    const double q = pfe_out ? pfe_quantile : 0.0;
    hjm_status st = enqueue_impl(ctx, n_paths, n_steps, dt, seed, path_offset, precision, hazard_rate, recovery, q,
                                 nullptr);
    if (st != HJM_OK) return st;
    return hjm_fetch_results(ctx, ee_out, pfe_out, cva_out);
}

hjm_status hjm_run_with_normals(hjm_ctx* ctx, int64_t n_paths, int32_t n_steps, double dt, const double* normals_host,
                                int32_t precision, double hazard_rate, double recovery, double pfe_quantile,
                                double* ee_out, double* pfe_out, double* cva_out)
{
    HJM_CHECK_CTX(ctx);
    if (!normals_host) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "normals must not be null");
    if (n_paths <= 0 || n_steps <= 0) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "n_paths and n_steps must be > 0");
    const size_t count = (size_t)n_paths * (size_t)n_steps * 3;
    if (count > ((size_t)1 << 33)) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "normals buffer too large");
    HJM_CUDA(ctx, cudaSetDevice(ctx->device));
    HJM_CUDA(ctx, ctx->ext_raw.ensure(sizeof(double) * count));
    HJM_CUDA(ctx, ctx->ext.ensure(sizeof(double) * count));
    HJM_CUDA(ctx, cudaMemcpyAsync(ctx->ext_raw.p, normals_host, sizeof(double) * count, cudaMemcpyHostToDevice,
                                  ctx->stream));
    HJM_CUDA(ctx, launch_transpose_normals((const double*)ctx->ext_raw.p, n_paths, n_steps, (double*)ctx->ext.p,
                                           ctx->stream));
    const double q = pfe_out ? pfe_quantile : 0.0;
    hjm_status st = enqueue_impl(ctx, n_paths, n_steps, dt, 0, 0, precision, hazard_rate, recovery, q,
                                 (const double*)ctx->ext.p);
    if (st != HJM_OK) return st;
    ctx->stat_launches += 1;
    ctx->stat_h2d += (int64_t)(sizeof(double) * count);
    return hjm_fetch_results(ctx, ee_out, pfe_out, cva_out);
}

hjm_status hjm_get_exposures(hjm_ctx* ctx, double* out_host, int64_t capacity)
{
    HJM_CHECK_CTX(ctx);
    if (!ctx->have_result || !ctx->last_stored)
        return fail(ctx, HJM_ERR_NOT_CONFIGURED,
                    "no stored exposures: run with a PFE quantile or after hjm_ctx_keep_exposures(ctx, 1)");
    const int64_t need = ctx->last_n_paths * (int64_t)ctx->last_n_dates;
    if (!out_host || capacity < need)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "exposure buffer holds %lld values, %lld needed",
                    (long long)capacity, (long long)need);
    HJM_CUDA(ctx, cudaSetDevice(ctx->device));
    HJM_CUDA(ctx, ctx->wide.ensure(sizeof(double) * (size_t)need));
    HJM_CUDA(ctx, launch_widen_exposures(ctx->estore.p, !ctx->last_mixed, ctx->last_ld, ctx->last_n_paths,
                                         ctx->last_n_dates, (double*)ctx->wide.p, ctx->stream));
    HJM_CUDA(ctx, cudaMemcpyAsync(out_host, ctx->wide.p, sizeof(double) * (size_t)need, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    HJM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HJM_OK;
}

hjm_status hjm_get_exposure_paths(hjm_ctx* ctx, int64_t path_begin, int64_t n, double* out_host)
{
    HJM_CHECK_CTX(ctx);
    if (!ctx->have_result || !ctx->last_stored)
        return fail(ctx, HJM_ERR_NOT_CONFIGURED,
                    "no stored exposures: run with a PFE quantile or after hjm_ctx_keep_exposures(ctx, 1)");
    if (!out_host || n <= 0 || path_begin < 0 || path_begin > ctx->last_n_paths - n)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "paths [%lld, %lld + %lld) outside the run's %lld paths",
                    (long long)path_begin, (long long)path_begin, (long long)n, (long long)ctx->last_n_paths);
    HJM_CUDA(ctx, cudaSetDevice(ctx->device));
    const size_t rows = (size_t)ctx->last_n_dates, cols = (size_t)n;
    const size_t es = ctx->last_mixed ? sizeof(float) : sizeof(double);
    const char* src = (const char*)ctx->estore.p + (size_t)path_begin * es;
    if (!ctx->last_mixed) {
        HJM_CUDA(ctx, cudaMemcpy2DAsync(out_host, cols * sizeof(double), src, (size_t)ctx->last_ld * es,
                                        cols * es, rows, cudaMemcpyDeviceToHost, ctx->stream));
        HJM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    } else {
        std::vector<float> tmp(rows * cols);
        HJM_CUDA(ctx, cudaMemcpy2DAsync(tmp.data(), cols * sizeof(float), src, (size_t)ctx->last_ld * es,
                                        cols * es, rows, cudaMemcpyDeviceToHost, ctx->stream));
        HJM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (size_t i = 0; i < rows * cols; ++i) out_host[i] = (double)tmp[i];
    }
    return HJM_OK;
}

// ---------------------------------------------------------------------------
// diagnostics
// ---------------------------------------------------------------------------
hjm_status hjm_dump_normals(hjm_ctx* ctx, int64_t n_paths, uint64_t path_offset, int32_t n_steps, uint64_t seed,
                            double* out_host)
{
    HJM_CHECK_CTX(ctx);
    if (n_paths <= 0 || n_steps <= 0 || !out_host)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "n_paths, n_steps must be > 0 and out non-null");
    const size_t count = (size_t)n_paths * (size_t)n_steps * 3;
    if (count > ((size_t)1 << 33)) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "normals buffer too large");
    HJM_CUDA(ctx, cudaSetDevice(ctx->device));
    HJM_CUDA(ctx, ctx->scratch.ensure(sizeof(double) * count));
    HJM_CUDA(ctx, launch_dump_normals(n_paths, path_offset, n_steps, (uint32_t)seed, (uint32_t)(seed >> 32),
                                      (double*)ctx->scratch.p, ctx->stream));
    HJM_CUDA(ctx, cudaMemcpyAsync(out_host, ctx->scratch.p, sizeof(double) * count, cudaMemcpyDeviceToHost,
                                  ctx->stream));
    HJM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HJM_OK;
}

hjm_status hjm_philox_words(hjm_ctx* ctx, int64_t n_paths, uint64_t path_offset, uint32_t step, uint64_t seed,
                            uint32_t* out_host)
{
    HJM_CHECK_CTX(ctx);
    if (n_paths <= 0 || n_paths > ((int64_t)1 << 28) || !out_host)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "n_paths must be in [1, 2^28] and out non-null");
    HJM_CUDA(ctx, cudaSetDevice(ctx->device));
    HJM_CUDA(ctx, ctx->scratch.ensure(sizeof(uint32_t) * 4 * (size_t)n_paths));
    HJM_CUDA(ctx, launch_philox_words(n_paths, path_offset, step, (uint32_t)seed, (uint32_t)(seed >> 32),
                                      (uint32_t*)ctx->scratch.p, ctx->stream));
    HJM_CUDA(ctx, cudaMemcpyAsync(out_host, ctx->scratch.p, sizeof(uint32_t) * 4 * (size_t)n_paths,
                                  cudaMemcpyDeviceToHost, ctx->stream));
    HJM_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    return HJM_OK;
}

hjm_status hjm_last_timings(hjm_ctx* ctx, double* ms_out)
{
    HJM_CHECK_CTX(ctx);
    if (!ms_out) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "ms_out must not be null");
    if (!ctx->have_result) return fail(ctx, HJM_ERR_NOT_CONFIGURED, "no valuation has been enqueued");
    HJM_CUDA(ctx, cudaEventSynchronize(ctx->ev[3]));
    float a = 0, b = 0, c = 0, d = 0;
    HJM_CUDA(ctx, cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[1]));
    HJM_CUDA(ctx, cudaEventElapsedTime(&b, ctx->ev[1], ctx->ev[2]));
    HJM_CUDA(ctx, cudaEventElapsedTime(&c, ctx->ev[2], ctx->ev[3]));
    HJM_CUDA(ctx, cudaEventElapsedTime(&d, ctx->ev[0], ctx->ev[3]));
    ms_out[0] = a;
    ms_out[1] = b;
    ms_out[2] = c;
    ms_out[3] = d;
    return HJM_OK;
}

hjm_status hjm_timing_history(hjm_ctx* ctx, int32_t n, double* ms_out)
{
    HJM_CHECK_CTX(ctx);
    if (!ms_out || n <= 0) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "need n > 0 and ms_out non-null");
    if (n > hjm_ctx::kRing || n > ctx->n_enqueued)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "history holds min(%d, %lld) valuations, %d requested",
                    hjm_ctx::kRing, (long long)ctx->n_enqueued, n);
    HJM_CUDA(ctx, cudaSetDevice(ctx->device));
    for (int i = 0; i < n; ++i) {
        const int64_t idx = ctx->n_enqueued - n + i;
        cudaEvent_t* q = ctx->ring[idx % hjm_ctx::kRing];
        HJM_CUDA(ctx, cudaEventSynchronize(q[3]));
        float a = 0, b = 0, c = 0, d = 0;
        HJM_CUDA(ctx, cudaEventElapsedTime(&a, q[0], q[1]));
        HJM_CUDA(ctx, cudaEventElapsedTime(&b, q[1], q[2]));
        HJM_CUDA(ctx, cudaEventElapsedTime(&c, q[2], q[3]));
        HJM_CUDA(ctx, cudaEventElapsedTime(&d, q[0], q[3]));
        ms_out[4 * i + 0] = a;
        ms_out[4 * i + 1] = b;
        ms_out[4 * i + 2] = c;
        ms_out[4 * i + 3] = d;
    }
    return HJM_OK;
}

hjm_status hjm_last_stats(hjm_ctx* ctx, int64_t* stats_out)
{
    HJM_CHECK_CTX(ctx);
    if (!stats_out) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "stats_out must not be null");
    stats_out[0] = ctx->stat_launches;
    stats_out[1] = ctx->stat_h2d;
    stats_out[2] = ctx->stat_d2h;
    return HJM_OK;
}

hjm_status hjm_measure_fma_peak(hjm_ctx* ctx, int32_t precision, double* tflops_out)
{
    HJM_CHECK_CTX(ctx);
    if (!tflops_out) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "tflops_out must not be null");
    HJM_CUDA(ctx, cudaSetDevice(ctx->device));
    HJM_CUDA(ctx, measure_fma_peak(precision == HJM_PRECISION_FP64, ctx->stream, ctx->n_sms, tflops_out));
    return HJM_OK;
}

// ---------------------------------------------------------------------------
// adjoint
// ---------------------------------------------------------------------------
hjm_status hjm_run_adjoint(hjm_ctx* ctx, int64_t n_paths, int32_t n_steps, double dt, uint64_t seed,
                           uint64_t path_offset, double hazard_rate, double recovery, int32_t checkpoint_every,
                           double* cva_out, double* dcva_dspot_out, double* dcva_ddrift_out,
                           double* dcva_dvolcoef_out)
{
    HJM_CHECK_CTX(ctx);
    RunShape sh;
    hjm_status st = check_run(ctx, n_paths, n_steps, dt, HJM_PRECISION_MIXED, hazard_rate, recovery, 0.0, sh);
    if (st != HJM_OK) return st;
    const bool pc = ctx->scheme == HJM_SCHEME_PREDICTOR_CORRECTOR;
    if (pc && checkpoint_every != 0)
        return fail(ctx, HJM_ERR_UNSUPPORTED,
                    "the predictor-corrector adjoint keeps the sampled states: checkpoint_every must be 0");
    if (checkpoint_every < 0 || checkpoint_every > sh.stride)
        return fail(ctx, HJM_ERR_UNSUPPORTED, "checkpoint_every %d: must be 0 (none) or in [1, %d] (the block length)",
                    checkpoint_every, sh.stride);
    if (dcva_dvolcoef_out && !ctx->have_poly)
        return fail(ctx, HJM_ERR_NOT_CONFIGURED,
                    "volatility-coefficient sensitivities need a polynomial market (hjm_set_market_poly)");
    const int nt = ctx->nt, B = sh.B;
    const int R = adjoint_columns(nt, B);
    // quadratic factors under the Euler step with the sampled states kept:
    // the response form's adjoint where the valuation's response form fits
    const int adj_ns = (!pc && checkpoint_every == 0 && use_poly_path(ctx) && ctx->remainder != HJM_REMAINDER_CONVECT)
                           ? mresp_run_slots(ctx, sh, dt)
                           : 0;
    const size_t smem = pc ? adjoint_pc_smem(nt, B)
                           : (adj_ns ? adjoint_resp_smem(B) : adjoint_smem(nt, B, checkpoint_every > 0));
    if (smem > 227 * 1024) return fail(ctx, HJM_ERR_UNSUPPORTED, "adjoint shared memory %zu B exceeds 227 KB", smem);
    HJM_CUDA(ctx, cudaSetDevice(ctx->device));
    const int64_t n_ctas = (n_paths + adjoint_cta() - 1) / adjoint_cta();
    const int64_t ld = (n_paths + 3) / 4 * 4;
    const int E = n_steps - sh.stride;
    const int K = checkpoint_every;
    const int S = K > 0 ? (E + K - 1) / K : 0;
    HJM_CUDA(ctx, ctx->partials.ensure(sizeof(double) * (size_t)n_ctas * R));
    HJM_CUDA(ctx, ctx->sums.ensure(sizeof(double) * kMaxTenor * 4));
    HJM_CUDA(ctx, ctx->result.ensure(sizeof(double) * kResLen));
    if (K > 0) {
        HJM_CUDA(ctx, ctx->ck_h.ensure(sizeof(float) * (size_t)S * (nt + 5) * (size_t)ld));
        HJM_CUDA(ctx, ctx->ck_a.ensure(sizeof(double) * (size_t)S * (size_t)ld));
    }
    AdjParams A;
    PcParams<float> Qp;
    FinalParams F;
    std::memset(&A, 0, sizeof(A));
    {
        PathParams<float> P;
        fill_params<float>(ctx, sh, n_paths, dt, seed, path_offset, hazard_rate, recovery, 0, false, P, F);
        if (pc)
            fill_pc<float>(ctx, sh, dt, P, Qp);
        else
            pack_mixed_params(nt, P, A.M);
    }
    A.ckpt_every = K;
    A.ck_ld = ld;
    cudaStream_t s = ctx->stream;
    ctx->ev = ctx->ring[ctx->n_enqueued % hjm_ctx::kRing];
    ctx->n_enqueued++;
    HJM_CUDA(ctx, cudaMemsetAsync(ctx->result.p, 0, sizeof(double) * kResLen, s));
    HJM_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
    if (pc) {
        HJM_CUDA(ctx, launch_adjoint_pc(nt, Qp, use_poly_path(ctx), (double*)ctx->partials.p, s));
    } else if (adj_ns) {
        st = ensure_mresp_table(ctx, s);
        if (st != HJM_OK) return st;
        HJM_CUDA(ctx, launch_adjoint_resp(A, adj_ns, (const float4*)ctx->mresp.p, (double*)ctx->partials.p, s));
        HJM_CUDA(ctx, cudaEventRecord(ctx->resp_used, s));
    } else {
        HJM_CUDA(ctx, launch_adjoint(nt, A, use_poly_path(ctx), (double*)ctx->partials.p,
                                     K > 0 ? (float*)ctx->ck_h.p : nullptr, K > 0 ? (double*)ctx->ck_a.p : nullptr, s));
    }
    HJM_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
    HJM_CUDA(ctx, launch_reduce((const double*)ctx->partials.p, n_ctas, R, (double*)ctx->sums.p, F,
                                (double*)ctx->result.p, s));
    HJM_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
    HJM_CUDA(ctx, cudaEventRecord(ctx->ev[3], s));
    ctx->stat_launches = 3;
    ctx->stat_h2d = (pc ? sizeof(PcParams<float>) : sizeof(AdjParams)) + sizeof(FinalParams);
    std::vector<double> res(kResLen), sums(R);
    HJM_CUDA(ctx, cudaMemcpyAsync(res.data(), ctx->result.p, sizeof(double) * kResLen, cudaMemcpyDeviceToHost, s));
    HJM_CUDA(ctx, cudaMemcpyAsync(sums.data(), ctx->sums.p, sizeof(double) * R, cudaMemcpyDeviceToHost, s));
    HJM_CUDA(ctx, cudaStreamSynchronize(s));
    ctx->stat_d2h = (int64_t)sizeof(double) * (kResLen + R);
    ctx->have_result = false;  // the exposure-valuation result buffers are not this run's
    const double inv_n = 1.0 / (double)n_paths;
    if (cva_out) {
        cva_out[HJM_CVA_VALUE] = res[kResCVA];
        cva_out[HJM_CVA_STDERR] = res[kResCVAStderr];
        cva_out[HJM_CVA_DHAZARD] = res[kResDCVADHazard];
    }
    // dCVA/dspot and dCVA/dmu: the path means of the per-date seeds through the
    // FP64 adjoint of the deterministic curve (p_n = spot for the first block,
    // p_n = A p_{n-1} + dt mu after; date i reads p_{n_i}[i] and sum_{n<=n_i} p_n[i]).
    // Predictor-corrector: p_n = A2 p_{n-1} + dt N mu with A2 = I + dt D + dt^2
    // D^2 / 2 and N = I + dt D / 2 (D the forward difference / dtau, backward
    // at the last tenor), so q <- A2^T q and dmu += dt N^T q.
    std::vector<double> xbar(B + 1, 0.0), abar(B + 1, 0.0);
    for (int i = 1; i <= B; ++i) {
        xbar[i] = sums[B + 3 + i - 1] * inv_n;
        abar[i] = sums[2 * B + 3 + i - 1] * inv_n;
    }
    std::vector<double> q(nt, 0.0), qn(nt), d2(nt), dmu(nt, 0.0), inj(nt, 0.0);
    const double c = dt / ctx->dtau;
    const int L = nt - 1;
    for (int n = n_steps - 1; n >= sh.stride - 1; --n) {
        if ((n + 1) % sh.stride == 0) {  // step n samples date i
            const int i = (n + 1) / sh.stride;
            inj[i] = abar[i];
            q[i] += xbar[i];
        }
        for (int t = 0; t < nt; ++t) q[t] += inj[t];
        if (n < sh.stride) break;  // q = adjoint of p_{stride-1} = spot
        if (pc) {
            auto DT = [&](const std::vector<double>& y, std::vector<double>& out) {
                for (int t = 0; t < nt; ++t) out[t] = 0.0;
                for (int r = 0; r < L; ++r) {
                    out[r] -= y[r];
                    out[r + 1] += y[r];
                }
                out[L - 1] -= y[L];
                out[L] += y[L];
                for (int t = 0; t < nt; ++t) out[t] /= ctx->dtau;
            };
            DT(q, qn);
            DT(qn, d2);
            for (int t = 0; t < nt; ++t) {
                dmu[t] += dt * (q[t] + 0.5 * dt * qn[t]);
                q[t] += dt * qn[t] + 0.5 * dt * dt * d2[t];
            }
            continue;
        }
        for (int t = 0; t < nt; ++t) dmu[t] += dt * q[t];
        qn[0] = (1.0 - c) * q[0];
        for (int t = 1; t <= L - 2; ++t) qn[t] = q[t] + c * (q[t - 1] - q[t]);
        qn[L - 1] = q[L - 1] + c * (q[L - 2] - q[L - 1]) - c * q[L];
        qn[L] = q[L] + c * (q[L] + q[L - 1]);
        q.swap(qn);
    }
    hjm_ctx::Report& r = ctx->rep;
    r = hjm_ctx::Report();
    r.valid = r.adjoint = true;
    r.n_paths = n_paths;
    r.n_steps = n_steps;
    r.n_dates = B + 1;
    r.nt = nt;
    r.precision = HJM_PRECISION_MIXED;
    r.vol_form = use_poly_path(ctx) ? vol_form_code(ctx) : 0;  // a cubic market runs the table step here
    r.remainder = adj_ns ? 2 : 1;
    r.scheme = ctx->scheme;
    r.ckpt = K;
    r.dt = dt;
    r.dtau = ctx->dtau;
    r.hazard = hazard_rate;
    r.recovery = recovery;
    r.seed = seed;
    r.path_offset = path_offset;
    r.cva = res[kResCVA];
    r.cva_stderr = res[kResCVAStderr];
    r.dhazard = res[kResDCVADHazard];
    r.dspot.resize(nt);
    for (int t = 0; t < nt; ++t) r.dspot[t] = q[t] + (double)(sh.stride - 1) * inj[t];
    r.ddrift = dmu;
    if (dcva_dspot_out)
        for (int t = 0; t < nt; ++t) dcva_dspot_out[t] = r.dspot[t];
    if (dcva_ddrift_out)
        for (int t = 0; t < nt; ++t) dcva_ddrift_out[t] = dmu[t];
    if (ctx->have_poly) {
        // diffusion part, then the trapezoid drift's dependence on the coefficients:
        // mu_i = sum_k sigma_k(tau_i) I_k(i), I_k(i) = sum_{j<=i} (sigma_k(tau_j)+sigma_k(tau_{j-1}))/2 dtau
        // d mu_i / d c_{k,d} = tau_i^d I_k(i) + sigma_k(tau_i) J_d(i),  J_d(i) = sum_{j<=i} (tau_j^d+tau_{j-1}^d)/2 dtau
        const double sq = std::sqrt(dt);
        for (int k = 0; k < HJM_N_FACTOR; ++k) {
            const double* sig = ctx->vol.data() + (size_t)k * nt;
            // diffusion: Euler, the columns are dCVA/d(sqrt(dt) c_{k,d}); the
            // predictor-corrector, dCVA/d(aS_k, aU_k, aW_k) of the N-projected
            // loadings aS = sqrt(dt) (c0 + c dtau c1 / 2 + c dtau^2 c2 / 2),
            // aU = sqrt(dt) (c1 + c dtau c2), aW = sqrt(dt) c2
            const double X0 = sums[3 * B + 3 + k * 3] * inv_n, X1 = sums[3 * B + 3 + k * 3 + 1] * inv_n,
                         X2 = sums[3 * B + 3 + k * 3 + 2] * inv_n;
            const double cd = c * ctx->dtau;
            const double diff[3] = {pc ? X0 : X0, pc ? 0.5 * cd * X0 + X1 : X1,
                                    pc ? 0.5 * cd * ctx->dtau * X0 + cd * X1 + X2 : X2};
            for (int d = 0; d < 3; ++d) {
                double v = sq * diff[d];
                double I = 0.0, J = 0.0;
                for (int i = 0; i < nt; ++i) {
                    const double ti = ctx->dtau * i;
                    if (i > 0) {
                        const double tp = ctx->dtau * (i - 1);
                        I += 0.5 * (sig[i] + sig[i - 1]) * ctx->dtau;
                        J += 0.5 * (std::pow(ti, d) + std::pow(tp, d)) * ctx->dtau;
                    }
                    v += dmu[i] * (std::pow(ti, d) * I + sig[i] * J);
                }
                r.dcoef[k * 3 + d] = v;
                if (dcva_dvolcoef_out) dcva_dvolcoef_out[k * 3 + d] = v;
            }
        }
        r.have_dcoef = true;
    }
    return HJM_OK;
}

// ---------------------------------------------------------------------------
// multi-level Monte Carlo
// ---------------------------------------------------------------------------
hjm_status hjm_run_mlmc(hjm_ctx* ctx, int32_t n_levels, const int64_t* n_paths, int32_t n_steps, double dt,
                        uint64_t seed, double hazard_rate, double recovery, double* ee_out, double* cva_out,
                        double* level_out)
{
    HJM_CHECK_CTX(ctx);
    if (n_levels < 1 || n_levels > HJM_MLMC_MAX_LEVELS || !n_paths)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "n_levels must be in [1, %d] with n_paths per level",
                    HJM_MLMC_MAX_LEVELS);
    const bool pc = ctx->scheme == HJM_SCHEME_PREDICTOR_CORRECTOR;
    for (int l = 0; l < n_levels; ++l)
        if (n_paths[l] <= 0 || n_paths[l] > ((int64_t)1 << 31))
            return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "level %d: n_paths %lld outside [1, 2^31]", l,
                        (long long)n_paths[l]);
    // validate every level's grid (dt / 2^l, n_steps 2^l) before launching anything
    std::vector<RunShape> shapes(n_levels);
    for (int l = 0; l < n_levels; ++l) {
        hjm_status st = check_run(ctx, n_paths[l], n_steps << l, dt / (double)(1 << l), HJM_PRECISION_MIXED,
                                  hazard_rate, recovery, 0.0, shapes[l]);
        if (st != HJM_OK) return st;
        if (l >= 1 && (pc ? mlmc_pc_smem(ctx->nt, shapes[l].B) : mlmc_smem(shapes[l].B)) > 227 * 1024)
            return fail(ctx, HJM_ERR_UNSUPPORTED, "level %d: shared memory exceeds 227 KB", l);
    }
    const int nt = ctx->nt;
    std::vector<double> ee(nt, 0.0), lev(4 * (size_t)n_levels, 0.0);
    double cva = 0.0, var = 0.0, dhaz = 0.0;
    // level 0: the plain mixed-precision valuation on the coarsest grid
    {
        double e0[kMaxTenor], c0[HJM_CVA_OUT_LEN];
        hjm_status st = enqueue_impl(ctx, n_paths[0], n_steps, dt, seed, 0, HJM_PRECISION_MIXED, hazard_rate,
                                     recovery, 0.0, nullptr);
        if (st != HJM_OK) return st;
        st = hjm_fetch_results(ctx, e0, nullptr, c0);
        if (st != HJM_OK) return st;
        float ms = 0.f;
        HJM_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[2]));
        for (int j = 0; j < nt; ++j) ee[j] += e0[j];
        cva += c0[HJM_CVA_VALUE];
        var += c0[HJM_CVA_STDERR] * c0[HJM_CVA_STDERR];
        dhaz += c0[HJM_CVA_DHAZARD];
        lev[0] = c0[HJM_CVA_VALUE];
        lev[1] = c0[HJM_CVA_STDERR];
        lev[2] = ms;
        lev[3] = (double)n_paths[0];
    }
    // levels >= 1: the coupled kernel; normals of level l from path index + l 2^40
    cudaStream_t s = ctx->stream;
    for (int l = 1; l < n_levels; ++l) {
        const RunShape& shf = shapes[l];
        const RunShape& shc = shapes[l - 1];
        const double dtf = dt / (double)(1 << l), dtc = dt / (double)(1 << (l - 1));
        const uint64_t offset = (uint64_t)l << 40;
        const int R = shf.B + 3;
        const int64_t n_ctas = (n_paths[l] + mlmc_cta() - 1) / mlmc_cta();
        HJM_CUDA(ctx, ctx->partials.ensure(sizeof(double) * (size_t)n_ctas * R));
        HJM_CUDA(ctx, ctx->sums.ensure(sizeof(double) * kMaxTenor * 4));
        HJM_CUDA(ctx, ctx->result.ensure(sizeof(double) * kResLen));
        MlmcParams Q;
        MlmcPcParams Qp;
        FinalParams F, Fc;
        {
            PathParams<float> P;
            fill_params<float>(ctx, shf, n_paths[l], dtf, seed, offset, hazard_rate, recovery, 0, false, P, F);
            if (pc)
                fill_pc<float>(ctx, shf, dtf, P, Qp.fine);
            else
                pack_mixed_params(nt, P, Q.fine);
            fill_params<float>(ctx, shc, n_paths[l], dtc, seed, offset, hazard_rate, recovery, 0, false, P, Fc);
            if (pc)
                fill_pc<float>(ctx, shc, dtc, P, Qp.coarse);
            else
                pack_mixed_params(nt, P, Q.coarse);
        }
        ctx->ev = ctx->ring[ctx->n_enqueued % hjm_ctx::kRing];
        ctx->n_enqueued++;
        HJM_CUDA(ctx, cudaMemsetAsync(ctx->result.p, 0, sizeof(double) * kResLen, s));
        HJM_CUDA(ctx, cudaEventRecord(ctx->ev[0], s));
        if (pc)
            HJM_CUDA(ctx, launch_mlmc_level_pc(nt, Qp, use_poly_path(ctx), (double*)ctx->partials.p, s));
        else
            HJM_CUDA(ctx, launch_mlmc_level(nt, Q, use_poly_path(ctx), (double*)ctx->partials.p, s));
        HJM_CUDA(ctx, cudaEventRecord(ctx->ev[1], s));
        HJM_CUDA(ctx, launch_reduce((const double*)ctx->partials.p, n_ctas, R, (double*)ctx->sums.p, F,
                                    (double*)ctx->result.p, s));
        HJM_CUDA(ctx, cudaEventRecord(ctx->ev[2], s));
        HJM_CUDA(ctx, cudaEventRecord(ctx->ev[3], s));
        double res[kResLen];
        HJM_CUDA(ctx, cudaMemcpyAsync(res, ctx->result.p, sizeof(res), cudaMemcpyDeviceToHost, s));
        HJM_CUDA(ctx, cudaStreamSynchronize(s));
        float ms = 0.f;
        HJM_CUDA(ctx, cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[2]));
        for (int j = 0; j < nt; ++j) ee[j] += res[kResEE + j];
        cva += res[kResCVA];
        var += res[kResCVAStderr] * res[kResCVAStderr];
        dhaz += res[kResDCVADHazard];
        lev[4 * l + 0] = res[kResCVA];
        lev[4 * l + 1] = res[kResCVAStderr];
        lev[4 * l + 2] = ms;
        lev[4 * l + 3] = (double)n_paths[l];
    }
    ctx->have_result = false;  // the result buffers hold the last level, not a valuation
    {
        // the report describes the estimate: the finest grid, all levels' paths
        hjm_ctx::Report& r = ctx->rep;
        r = hjm_ctx::Report();
        r.valid = true;
        int64_t total = 0;
        for (int l = 0; l < n_levels; ++l) total += n_paths[l];
        r.n_paths = total;
        r.n_steps = n_steps << (n_levels - 1);
        r.dt = dt / (double)(1 << (n_levels - 1));
        r.n_dates = shapes[0].B + 1;
        r.nt = nt;
        r.precision = HJM_PRECISION_MIXED;
        r.vol_form = use_poly_path(ctx) ? vol_form_code(ctx) : 0;  // a cubic market runs the table step here
        r.remainder = 1;
        r.scheme = ctx->scheme;
        r.dtau = ctx->dtau;
        r.hazard = hazard_rate;
        r.recovery = recovery;
        r.seed = seed;
        r.ee = ee;
        r.cva = cva;
        r.cva_stderr = std::sqrt(var);
        r.dhazard = dhaz;
        r.levels = lev;
    }
    if (ee_out)
        for (int j = 0; j < nt; ++j) ee_out[j] = ee[j];
    if (cva_out) {
        cva_out[HJM_CVA_VALUE] = cva;
        cva_out[HJM_CVA_STDERR] = std::sqrt(var);
        cva_out[HJM_CVA_DHAZARD] = dhaz;
    }
    if (level_out)
        for (size_t q = 0; q < lev.size(); ++q) level_out[q] = lev[q];
    return HJM_OK;
}

// ---------------------------------------------------------------------------
// report
// ---------------------------------------------------------------------------
static void put_array(FILE* f, const char* name, const std::vector<double>& v, bool comma = true)
{
    std::fprintf(f, "  \"%s\": [", name);
    for (size_t i = 0; i < v.size(); ++i) std::fprintf(f, "%s%.17g", i ? ", " : "", v[i]);
    std::fprintf(f, "]%s\n", comma ? "," : "");
}

hjm_status hjm_write_report(hjm_ctx* ctx, const char* path, int32_t format)
{
    HJM_CHECK_CTX(ctx);
    const hjm_ctx::Report& r = ctx->rep;
    if (!r.valid) return fail(ctx, HJM_ERR_NOT_CONFIGURED, "no valuation fetched and no adjoint run yet");
    if (!path) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "path must not be null");
    if (format != HJM_REPORT_JSON && format != HJM_REPORT_CSV)
        return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "unknown report format %d", format);
    FILE* f = std::fopen(path, "w");
    if (!f) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "cannot open %s for writing", path);
    static const char* kForms[] = {"table", "poly", "poly_tri", "cubic_resid"};
    static const char* kRemainders[] = {"none", "convect", "response"};
    std::vector<double> dates(r.nt);
    for (int j = 0; j < r.nt; ++j) dates[j] = r.dtau * j;
    const char* prec = r.precision == HJM_PRECISION_FP64 ? "fp64" : "mixed";
    if (format == HJM_REPORT_JSON) {
        std::fprintf(f, "{\n  \"engine\": \"%s\",\n", hjm_version());
        std::fprintf(f, "  \"kind\": \"%s\",\n", r.adjoint ? "adjoint" : r.levels.empty() ? "valuation" : "mlmc");
        if (!r.levels.empty()) {
            std::fprintf(f, "  \"levels\": [");
            for (size_t l = 0; l < r.levels.size() / 4; ++l)
                std::fprintf(f, "%s{\"cva_diff\": %.17g, \"stderr\": %.17g, \"ms\": %.17g, \"n_paths\": %.0f}",
                             l ? ", " : "", r.levels[4 * l], r.levels[4 * l + 1], r.levels[4 * l + 2],
                             r.levels[4 * l + 3]);
            std::fprintf(f, "],\n");
        }
        std::fprintf(f,
                     "  \"run\": {\"n_paths\": %lld, \"n_steps\": %d, \"dt\": %.17g, \"dtau\": %.17g, "
                     "\"n_tenor\": %d, \"sampled_dates\": %d, \"seed\": %llu, \"path_offset\": %llu, "
                     "\"precision\": \"%s\", \"vol_form\": \"%s\", \"hazard\": %.17g, \"recovery\": %.17g, "
                     "\"pfe_quantile\": %.17g, \"checkpoint_every\": %d, \"external_normals\": %s, "
                     "\"scheme\": \"%s\", \"remainder\": \"%s\"},\n",
                     (long long)r.n_paths, r.n_steps, r.dt, r.dtau, r.nt, r.n_dates - 1, (unsigned long long)r.seed,
                     (unsigned long long)r.path_offset, prec, kForms[r.vol_form], r.hazard, r.recovery,
                     r.pfe ? r.pfe_q : 0.0, r.ckpt, r.external_normals ? "true" : "false",
                     r.scheme == HJM_SCHEME_PREDICTOR_CORRECTOR ? "predictor_corrector" : "euler",
                     kRemainders[r.remainder]);
        std::fprintf(f, "  \"cva\": %.17g,\n  \"cva_stderr\": %.17g,\n  \"dcva_dhazard\": %.17g,\n", r.cva,
                     r.cva_stderr, r.dhazard);
        put_array(f, "dates", dates);
        if (r.adjoint) {
            put_array(f, "dcva_dspot", r.dspot);
            std::vector<double> dc(r.dcoef, r.dcoef + HJM_N_VOL_COEF);
            put_array(f, "dcva_dvolcoef", dc, true);
            put_array(f, "dcva_ddrift", r.ddrift, false);
        } else {
            put_array(f, "ee", r.ee, r.pfe);
            if (r.pfe) put_array(f, "pfe", r.pfe_v, false);
        }
        std::fprintf(f, "}\n");
    } else {
        std::fprintf(f, "# %s %s\n", hjm_version(),
                     r.adjoint ? "adjoint" : r.levels.empty() ? "valuation" : "mlmc");
        for (size_t l = 0; l < r.levels.size() / 4; ++l)
            std::fprintf(f, "# level %zu: cva_diff %.17g stderr %.17g ms %.17g n_paths %.0f\n", l, r.levels[4 * l],
                         r.levels[4 * l + 1], r.levels[4 * l + 2], r.levels[4 * l + 3]);
        std::fprintf(f, "key,value\n");
        std::fprintf(f,
                     "n_paths,%lld\nn_steps,%d\ndt,%.17g\ndtau,%.17g\nseed,%llu\nprecision,%s\nvol_form,%s\n"
                     "scheme,%s\nremainder,%s\n",
                     (long long)r.n_paths, r.n_steps, r.dt, r.dtau, (unsigned long long)r.seed, prec,
                     kForms[r.vol_form], r.scheme == HJM_SCHEME_PREDICTOR_CORRECTOR ? "predictor_corrector" : "euler",
                     kRemainders[r.remainder]);
        std::fprintf(f, "hazard,%.17g\nrecovery,%.17g\ncva,%.17g\ncva_stderr,%.17g\ndcva_dhazard,%.17g\n", r.hazard,
                     r.recovery, r.cva, r.cva_stderr, r.dhazard);
        if (r.adjoint) {
            for (int q = 0; q < HJM_N_VOL_COEF; ++q)
                std::fprintf(f, "dcva_dvolcoef_%d%d,%.17g\n", q / 3, q % 3, r.dcoef[q]);
            std::fprintf(f, "tenor,t,dcva_dspot,dcva_ddrift\n");
            for (int j = 0; j < r.nt; ++j)
                std::fprintf(f, "%d,%.17g,%.17g,%.17g\n", j, dates[j], r.dspot[j], r.ddrift[j]);
        } else {
            std::fprintf(f, "date,t,ee,pfe\n");
            for (int j = 0; j < r.nt; ++j)
                std::fprintf(f, "%d,%.17g,%.17g,%.17g\n", j, dates[j], r.ee[j], r.pfe ? r.pfe_v[j] : 0.0);
        }
    }
    const bool ok = std::fclose(f) == 0;
    if (!ok) return fail(ctx, HJM_ERR_INVALID_ARGUMENT, "writing %s failed", path);
    return HJM_OK;
}

