// hjm_kernels.h -- host-side launchers of the device kernels (internal).
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

#include "hjm_device.cuh"

namespace hjm {

// Threads (paths) per CTA of the FP64 path kernels
constexpr int kFp64Cta = 64;

// Device result block (doubles)
constexpr int kResEE = 0;                       // [kMaxTenor]
constexpr int kResPFE = kMaxTenor;              // [kMaxTenor]
constexpr int kResCVA = 2 * kMaxTenor;
constexpr int kResCVAStderr = kResCVA + 1;
constexpr int kResDCVADHazard = kResCVA + 2;
constexpr int kResCVAPathMean = kResCVA + 3;    // mean of per-path CVA contributions
constexpr int kResLen = kResCVA + 8;

struct FinalParams {
    double cvaw[kMaxTenor];    // CVA weights per date
    double dcvaw[kMaxTenor];   // d(weights)/d(hazard)
    int64_t n_paths;
    int n_blocks;
};

struct SelState {
    uint64_t prefix, mask, k;
    uint32_t count;  // candidates matching the prefix after the last pass
    uint32_t stage;  // 0: global passes; 1: to compact and rank; 2: done
};
// Candidates of a date ranked in shared memory by the PFE selection.
constexpr int kPfeCap = 2048;

// Mixed-precision path kernel parameters: the FP32 parameter block plus the
// volatility coefficients packed in tenor pairs {tenor p, tenor p + ceil(NT/2)}
// for the packed FP32x2 FMA (two tenors per instruction).
struct MixedParams {
    PathParams<float> P;
    float2 svp[kFactors][kMaxTenor / 2];
    float2 rp;  // {rr, rr}: the growth-scaled upwind coefficient
    // polynomial volatility in FP32: sqrt(dt) sigma_k(T) = sum_d svcf[k][d] T^d
    // (+ svcx[k] T^3 for a cubic, T then the tenor minus the basis centre)
    float svcf[kFactors][3];
    float k1f, k2f;  // c dtau, c dtau^2
    float svcx[kFactors];
    float k3f;       // c dtau^3
    float src3f;     // 3 (T_L - centre): the cubic's share of the remainder's source
};


// Volatility forms of the FP64 path kernel.
constexpr int kFormTable = 0;    // volatility table PathParams::sv
constexpr int kFormPoly = 1;     // factors quadratic in T, PathParams::svc
constexpr int kFormPolyTri = 2;  // ... with factor k of degree <= k

// The convected FP64 path kernel.  poly: the volatility factors are
// polynomials of degree <= 2 in T (PathParams::svc), else the table step.
// (The response forms of the Euler step are in hjm_eresp.h.)
cudaError_t launch_path_fp64(int nt, const PathParams<double>& P, bool poly, const double* ext, double* partials,
                             double* estore, cudaStream_t s);
int response_max_dates();
// The response form of the volatility-table step (FP64 accuracy, either
// scheme: the table carries the scheme): vresp from launch_response_table_vol
// with the kernel's loadings sv [kFactors][kMaxTenor] (PathParams::sv); one
// launch per window of at most max_slots dates (16, or 24 for one launch up
// to 24 dates; vresp_windows of them), carry [2][n_paths] doubles when there
// is more than one; *launches: kernels enqueued.
cudaError_t launch_path_fp64_vresp(int nt, const PathParams<double>& P, const float4* vresp, const double* ext,
                                   double* partials, double* estore, double* carry, cudaStream_t s,
                                   int* launches = nullptr, int max_slots = 16);
int vresp_windows(int n_blocks, int max_slots = 16);
int vresp_row(int n_blocks);                                // slots per table row
size_t response_table_vol_elems(int stride, int n_blocks);  // float4 entries
cudaError_t launch_response_table_vol(int nt, double c, int stride, int n_blocks, bool pc, const double* sv,
                                      float4* vresp, cudaStream_t s);
// cub: the cubic polynomial form (MixedParams::svcx, k3f, src3f; P.tau the
// tenors minus the basis centre), which implies poly
cudaError_t launch_path_mixed(int nt, const MixedParams& M, bool poly, const double* ext, double* partials,
                              float* estore, cudaStream_t s, bool cub = false);
void pack_mixed_params(int nt, const PathParams<float>& P, MixedParams& M);
// The response form of the mixed-precision Euler step (hjm_mresp.cu):
// polynomial factors (cub: the cubic form), the remainder as FP32
// impulse-response sums at the dates it reaches.  mresp_slots: the date
// slots of the run shape, 8 or 16, or 0 when the dates whose responses count
// do not fit 16 (the run then convects); launch_mresp_table: the table on
// the stream (rows b stride + s of ns / 2 float4, each two {kappa G,
// kappa CG} pairs; mresp_table_elems float4).
// pc: the predictor-corrector step's remainder (its parts then run the same
// kernel with the N-projected loadings aS, aU, aW as the coefficients of 1,
// T, T^2 and k2f = (c + c^2) dtau^2; not for a run whose last date samples
// the last tenor)
int mresp_slots(int nt, double c, double dtau, int stride, int n_blocks, bool pc = false);
size_t mresp_table_elems(int stride, int n_blocks, int ns);
cudaError_t launch_mresp_table(int nt, double c, double dtau, int stride, int n_blocks, int ns, bool pc,
                               float4* table, cudaStream_t s);
size_t mresp_smem_bytes(int n_blocks);
// paths per CTA: kCta, as launch_path_mixed's table form (path_cta)
cudaError_t launch_path_mixed_resp(const MixedParams& M, int ns, bool cub, const float4* table, const double* ext,
                                   double* partials, float* estore, cudaStream_t s);
bool path_tenor_supported(int nt);
size_t path_smem(int nt, int n_blocks, bool mixed);
// paths per CTA of the Euler path kernel of a run (one partial-sum row each):
// FP64 64; mixed 128, or 64 with the compact sums (polynomial factors, many dates)
int path_cta(bool mixed, int nt, int n_blocks, bool poly);

cudaError_t launch_reduce(const double* partials, int64_t n_rows, int R, double* sums, const FinalParams& F,
                          double* result, cudaStream_t s);
// scratch: pfe_scratch_bytes() of device memory (histograms, counters,
// candidate buffers).
size_t pfe_scratch_bytes();
cudaError_t launch_pfe(const void* estore, bool fp64_keys, int64_t ld, int64_t n_paths, int n_dates, uint64_t k0,
                       SelState* st, void* scratch, double* result, int n_sms, cudaStream_t s);
cudaError_t launch_dump_normals(int64_t n_paths, uint64_t path_offset, int n_steps, uint32_t k0, uint32_t k1,
                                double* out, cudaStream_t s);
cudaError_t launch_philox_words(int64_t n_paths, uint64_t path_offset, uint32_t step, uint32_t k0, uint32_t k1,
                                uint32_t* out, cudaStream_t s);
cudaError_t launch_transpose_normals(const double* in, int64_t n_paths, int n_steps, double* out, cudaStream_t s);
cudaError_t launch_widen_exposures(const void* in, bool fp64, int64_t ld, int64_t n_paths, int n_dates, double* out,
                                   cudaStream_t s);
cudaError_t measure_fma_peak(bool fp64, cudaStream_t s, int n_sms, double* tflops);

// Predictor-corrector kernel parameters: the path parameters (loadings
// N sqrt(dt) sigma, the PC deterministic curve, growth scales with base =
// 1 + r1 + r2) plus the stencil and the effective recovery coefficients.
template <typename T>
struct PcParams {
    PathParams<T> P;
    T r1, r2;              // a1 / a0, a2 / a0 (rounded once)
    T a0e, a1e, a2e, ce;   // effective scheme: 1/base, r1/base, r2/base, (r1 + 2 r2)/base
    T inv_1ma0, inv_ce;    // 1 / (1 - a0e), 1 / ce
    // polynomial form (factors of degree <= 2, PathParams::svc): h = S + U T +
    // W T^2 + remainder, with the noise N xi projected onto S, U, W and
    // last-tenor sources for the remainder
    T aS[kFactors], aU[kFactors], aW[kFactors];  // noise loadings of S, U, W
    T k1, k2p, k1x2;       // c dtau, (c + c^2) dtau^2, 2 c dtau
    T wL1, wL, gL;         // sources: -c^2 dtau^2 W at L-1; -(2c + c^2) dtau^2 W - c dtau^2 gamma at L
};

// The predictor-corrector's convected kernels (the FP64 response form of its
// decomposition runs in hjm_eresp.cu)
cudaError_t launch_path_pc(int nt, const PcParams<double>& Q, bool poly, const double* ext, double* partials,
                           double* estore, cudaStream_t s);
cudaError_t launch_path_pc(int nt, const PcParams<float>& Q, bool poly, const double* ext, double* partials,
                           float* estore, cudaStream_t s);
size_t pc_smem(int nt, int n_blocks, bool mixed);
int pc_cta();

// Multi-level Monte Carlo: the coupled level kernel's two parameter blocks
// (the fine grid, and the coarse grid with half the steps per block).
struct MlmcParams {
    MixedParams fine;
    MixedParams coarse;
};
cudaError_t launch_mlmc_level(int nt, const MlmcParams& Q, bool poly, double* partials, cudaStream_t s);
// ... and the predictor-corrector's (fine and coarse PcParams)
struct MlmcPcParams {
    PcParams<float> fine;
    PcParams<float> coarse;
};
cudaError_t launch_mlmc_level_pc(int nt, const MlmcPcParams& Q, bool poly, double* partials, cudaStream_t s);
size_t mlmc_pc_smem(int nt, int n_blocks);
size_t mlmc_smem(int n_blocks);
int mlmc_cta();

// Adjoint kernel parameters: the mixed-precision path parameters plus the
// checkpoint layout.
struct AdjParams {
    MixedParams M;
    int ckpt_every;                // 0: no checkpoints; else K in [1, stride]
    int64_t ck_ld;                 // row stride of the checkpoint arrays
};
size_t adjoint_smem(int nt, int n_blocks, bool ckpt);  // ckpt: the checkpoint mode's layout
int adjoint_columns(int nt, int n_blocks);
int adjoint_cta();  // paths per CTA of the adjoint kernel (one partial-sum row each)
cudaError_t launch_adjoint(int nt, const AdjParams& A, bool poly, double* partials, float* ck_h, double* ck_a,
                           cudaStream_t s);
// the adjoint in the response form (Euler, quadratic factors, sampled states
// kept): the mixed response form's forward pass and table (mresp_slots'
// ns slots), the same partial-sum columns as launch_adjoint
size_t adjoint_resp_smem(int n_blocks);
cudaError_t launch_adjoint_resp(const AdjParams& A, int ns, const float4* table, double* partials, cudaStream_t s);
// the predictor-corrector adjoint (sampled states kept; same partial-sum columns
// as launch_adjoint, the coefficient columns gather phi_k (M0, M1, M2 + gL g[L]))
size_t adjoint_pc_smem(int nt, int n_blocks);
cudaError_t launch_adjoint_pc(int nt, const PcParams<float>& Q, bool poly, double* partials, cudaStream_t s);

}  // namespace hjm
