// hjm_forward.cu -- fused Monte Carlo path kernel, reductions and PFE selection.
//
// One launch of path_kernel replaces the reference's whole GPU pipeline
// (simulation_gpu.cu:956-1179): cuRAND normal buffer (:1057-1071), 2,500
// single-step launches each followed by cudaDeviceSynchronize (:724-796, or
// the 50-step kernel4 variant :471-669), the exposure kernel (:803-882) and
// the cuBLAS gemv column sum (:889-933).  One thread owns one Monte Carlo
// path for its whole life: the curve sits in registers, normals come from
// Philox in registers, the numeraire of each 0.5y block end is priced on the
// spot, and the per-path exposure profile is reduced inside the CTA.
//
// Semantics follow the reference CPU path (simulation_cpu.h:188-296), which
// the reference's shared-memory GPU kernel also reproduces (xls RMSE 0.0):
//   * block 0 (steps 0..stride-1) holds the curve at spot (simulation_cpu.h:212);
//   * after block b the numeraire of tenor i = b+1 is sampled: forward f[i] and
//     discount exp(-dt * sum of f[i] over all steps so far) (simulation_cpu.h:248-250);
//   * cash flow of date i: D_i * N * alpha_i * (L_i - K), L = m (e^{f/m} - 1);
//     exposure E_j = max(sum_{i>j} cf_i, 0) (simulation_cpu.h:279-295).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "hjm_device.cuh"
#include "hjm_eresp.h"
#include "hjm_kernels.h"
#include "hjm_pairs.cuh"
#include "hjm_resp.cuh"
#include "hjm_epilogue.cuh"

namespace hjm {

// Shared-memory layout of the FP64 path kernel (dynamic), per CTA of
// kFp64Cta threads, column tid private to its thread until the epilogue:
//   cf_s   [B+1] double   cash flows of the sampled dates
//   acc_s  [B+1] double   FP64 discount sums of the stochastic part per tenor
//   work_s [2(B+2)] double  curve at block start / end, then exposures
//   red_s  [2 * kFp64Cta/32] double  CVA statistics

__host__ __device__ inline size_t path_smem_bytes(int nt, int n_blocks, bool mixed)
{
    (void)nt;
    (void)mixed;
    const size_t rows = (size_t)n_blocks + 1;
    size_t b = rows * kFp64Cta * 8;  // cf_s
    b += rows * kFp64Cta * 8;        // acc_s
    b = (b + 127) & ~(size_t)127;
    b += 2 * (rows + 1) * kFp64Cta * 8;  // work_s
    b += 2 * (kFp64Cta / 32) * 8;        // red_s
    return b;
}

// Discount sums by block-sum recovery.  Over one block of Euler steps
// n = n0 .. n0+stride-1 the states h_n = A h_{n-1} + xi_n sum to
//     (I - A) H = sum_n xi_n - A (h_end - h_start),   H = sum_n h_n,
// and (I - A) H [t] = c (H[t] - H[t+1]) for t below the last tenor.  So with
// one tenor accumulated directly (H[B], the last tenor still to be sampled),
//     H[t] = H[t+1] + (Xi[t] - (A d)[t]) / c,  d = h_end - h_start,
// gives every block sum the discount needs in O(B) FP64 operations per block
// instead of one FP64 addition per tenor per step (the FP64 pipe is the bound).
// Exact in exact arithmetic; in FP64 the recovered sums differ from step-by-
// step accumulation by ~1e-14 relative.
//
// Polynomial volatility (POLY).  When sqrt(dt) sigma_k(T) = sum_d svc[k][d] T^d
// with degree <= 2, the noise of a step is xi = alpha + beta T + gamma T^2 and
// the convection operator maps that basis into itself up to one last-tenor
// term:  A 1 = 1,  A T = T + c dtau 1,  A T^2 = T^2 + 2 c dtau T + c dtau^2 1
// - 2 c dtau^2 e_L.  Writing h = S 1 + U T + W T^2 + hc, the Euler step becomes
//     S <- S + c dtau U + c dtau^2 W + alpha,   U <- U + 2 c dtau W + beta,
//     W <- W + gamma,   hc <- A hc - 2 c dtau^2 W e_L   (old U, W on the right),
// exact in exact arithmetic: the curve is advanced in full, with the
// convection of hc per tenor instead of 5 operations, plus a dozen per step.
// With the growth scaling of PathParams (v = h / (1-c)^j) the convection is
// one FMA per tenor, and the table form four.
// FORM: kFormTable (volatility table), kFormPoly (quadratic factors) or
// kFormPolyTri (factor k of degree <= k, as the synthetic workloads' factors: the noise
// projection then skips the three zero coefficients).
template <int NT, bool EXT, int FORM>
__global__ void __launch_bounds__(kFp64Cta, 4)
    path_kernel_fp64(const __grid_constant__ PathParams<double> P, const double* __restrict__ ext,
                     double* __restrict__ partials, double* __restrict__ estore)
{
    constexpr int kCta = kFp64Cta;
    constexpr int L = NT - 1;
    constexpr bool POLY = FORM != kFormTable;
    constexpr bool TRI = FORM == kFormPolyTri;
    constexpr int kGroup = 8;                      // dead-tenor skipping granularity (4 measured slower)
    constexpr int kGroups = (L + kGroup - 1) / kGroup;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const int rows = B + 1;
    double* cf_s = reinterpret_cast<double*>(smem);
    double* acc_s = cf_s + (size_t)rows * kCta;
    size_t off = ((size_t)rows * kCta * 16 + 127) & ~(size_t)127;
    double* work_s = reinterpret_cast<double*>(smem + off);
    double* red_s = work_s + (size_t)2 * (rows + 1) * kCta;

    const int64_t cta_base = (int64_t)blockIdx.x * kCta;
    const int64_t lp = cta_base + tid;            // path index within this launch
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;

    // stochastic part of the curve (POLY: its convected remainder hc); zero
    // through block 0 (spot hold)
    double h[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) h[t] = 0.0;
    double S = 0.0, U = 0.0, W = 0.0;  // POLY: parallel, tilt and curvature parts
    for (int i = 0; i < rows; ++i) acc_s[i * kCta + tid] = 0.0;
    double* hs_s = work_s;
    double* he_s = work_s + (size_t)(rows + 1) * kCta;
    for (int t = 0; t <= B + 1; ++t) hs_s[t * kCta + tid] = 0.0;

    double g = 1.0;  // the kernel holds v; h = g v
    auto value_at = [&](int i) -> double {
        double v = g * select_reg<NT, double>(h, i);
        if (POLY) v += fma(P.tau[i], fma(P.tau[i], W, U), S);
        return v;
    };
    // price date i from the sampled numeraire (x_i, D_i)
    auto sample = [&](int i) {
        const double x = P.psamp[i] + value_at(i);
        const double a = P.psum[i] + acc_s[i * kCta + tid];
        const double D = exp(-a * P.dt);
        const double Lb = P.m * (exp(x * P.inv_m) - 1.0);
        cf_s[i * kCta + tid] = D * (P.payA[i] * Lb - P.payB[i]);
    };

    sample(1);
    const double c = P.c, rr = P.rr;
    for (int b = 1; b < B; ++b) {
        double f0 = 0.0, f1 = 0.0, f2 = 0.0;  // block sums of phi_k
        double sS = 0.0, sU = 0.0, sW = 0.0;  // POLY: block sums of S, U, W
        // anchor: hb = sum_s h_s[B] = g_end * Tb with Tb <- (1 + rr) Tb + v[B]
        // (g_s = g_end (1 + rr)^(stride - s)), one FMA per step
        double Tb = 0.0;
        double ig = P.igblk[b];          // table form: (1 + rr)^n'
        // tenors <= b are never read again (date b was sampled; the upwind step
        // carries information from high to low tenors only): their groups of
        // kGroup tenors are skipped, which changes no output bit
        const int live = b + 1;
        double mig = P.m2k2 * P.igblk[b];  // polynomial form: -2 c dtau^2 (1 + rr)^n'
        for (int s = 0; s < P.stride; ++s) {
            const int n = b * P.stride + s;
            double phi0, phi1, phi2;
            draw_phi<double, EXT>(ext, gpath, active ? lp : 0, P.n_paths, n, P.rk0, P.rk1, phi0, phi1, phi2);
            // in place, ascending (h[t+1] is still the old value); the last
            // tenor, which reads h[L-1], first
            if constexpr (POLY) {
                // the noise projection folded into the updates of S, U, W:
                // S' = S + c dtau U + c dtau^2 W + sum_k svc[k][0] phi_k, etc.
                // (old U, W on the right; factor k of degree <= k drops 3 terms)
                mig *= P.ip;
                const double hl = fma(mig, W, fma(rr, fma(2.0, h[L], -h[L - 1]), h[L]));  // + scaled source
#pragma unroll
                for (int gi = 0; gi < kGroups; ++gi) {
                    // uniform: skip groups of dead tenors, and (polynomial form)
                    // the exact zeros below the remainder's front: driven only
                    // at the last tenor from zero, after k steps it is nonzero
                    // on tenors >= L - k only
                    const int front = L - 1 - ((b - 1) * P.stride + s);
                    if (kGroup * gi + kGroup > (live > front ? live : front)) {
#pragma unroll
                        for (int j = 0; j < kGroup; ++j) {
                            const int t = kGroup * gi + j;
                            if (t < L) h[t] = fma(rr, h[t + 1], h[t]);
                        }
                    }
                }
                h[L] = hl;
                double Sn = fma(P.svc[0][0], phi0, fma(P.k2, W, fma(P.k1, U, S)));
                Sn = fma(P.svc[2][0], phi2, fma(P.svc[1][0], phi1, Sn));
                double Un = fma(P.svc[2][1], phi2, fma(P.svc[1][1], phi1, fma(2.0 * P.k1, W, U)));
                double Wn = fma(P.svc[2][2], phi2, W);
                if constexpr (!TRI) {
                    Un = fma(P.svc[0][1], phi0, Un);
                    Wn = fma(P.svc[1][2], phi1, fma(P.svc[0][2], phi0, Wn));
                }
                S = Sn;
                U = Un;
                W = Wn;
                sS += S;
                sU += U;
                sW += W;
            } else {
                ig *= P.ip;
                const double p0 = phi0 * ig, p1 = phi1 * ig, p2 = phi2 * ig;
                double xl = fma(P.sv[0][L], p0, h[L]);
                xl = fma(P.sv[1][L], p1, xl);
                xl = fma(P.sv[2][L], p2, xl);
                const double hl = fma(rr, fma(2.0, h[L], -h[L - 1]), xl);
#pragma unroll
                for (int gi = 0; gi < kGroups; ++gi) {
                    if (kGroup * gi + kGroup > live) {
#pragma unroll
                        for (int j = 0; j < kGroup; ++j) {
                            const int t = kGroup * gi + j;
                            if (t < L) {
                                double x = fma(P.sv[0][t], p0, h[t]);
                                x = fma(P.sv[1][t], p1, x);
                                x = fma(P.sv[2][t], p2, x);
                                h[t] = fma(rr, h[t + 1], x);
                            }
                        }
                    }
                }
                h[L] = hl;
                f0 += phi0;
                f1 += phi1;
                f2 += phi2;
            }
            Tb = fma(P.ip, Tb, select_reg<NT, double>(h, B));
        }
        g = P.gblk[b + 1];  // (1 + rr)^-(b stride): the scale at the block end
        const double hb = g * Tb;
#pragma unroll
        for (int t = 0; t < NT; ++t)
            if (t <= B + 1) he_s[t * kCta + tid] = g * h[t];
        auto poly_part = [&](int t) -> double {
            return POLY ? fma(P.tau[t], fma(P.tau[t], sW, sU), sS) : 0.0;
        };
        double Hn = hb;
        acc_s[B * kCta + tid] += Hn + poly_part(B);
        double dn = he_s[B * kCta + tid] - hs_s[B * kCta + tid];
        for (int t = B - 1; t > b; --t) {
            const double d = he_s[t * kCta + tid] - hs_s[t * kCta + tid];
            const double xi = POLY ? 0.0 : fma(P.sv[2][t], f2, fma(P.sv[1][t], f1, P.sv[0][t] * f0));
            const double ad = fma(c, dn - d, d);
            Hn = fma(xi - ad, P.inv_c, Hn);
            acc_s[t * kCta + tid] += Hn + poly_part(t);
            dn = d;
        }
        double* tmp = hs_s;
        hs_s = he_s;
        he_s = tmp;
        sample(b + 1);
    }

    fp64_epilogue<kCta>(P, cf_s, work_s, red_s, partials, estore, cta_base, active);
}

// Response form of the volatility-table step (FP64 accuracy, any factor
// shapes, both time schemes).  Without a polynomial part the whole
// stochastic curve is driven by the injected noise: h_n = A h_{n-1} + S phi_n
// (A the upwind step, or the predictor-corrector's A2 with the loadings S
// N-projected), so at date j's tenor after step K
//     h_K[j] = sum_{n<=K} sum_k phi_{n,k} R_jk(K - n),   R_jk(l) = (A^l S_k)[j],
// and its running sum likewise with CR_jk(l) = sum_{r<=l} R_jk(r).  Per step
// and date still to be sampled, three terms (the factors) into {value,
// running sum}, on coefficients read from the table (response_table_vol_kernel),
// in place of four FMAs per live tenor and the block-end recovery.  The sums
// run in double-FP32 on the FP32 pipe: the table holds each coefficient as
// FP32 hi + lo (48 bits), a generator normal is exact in FP32 (an external
// FP64 normal is split hi + lo), the product's leading term is exact by FMA
// and Knuth's two-sum adds it (df_acc_w / df_acc), and the pairs are
// renormalised after every step's three terms, so each addition rounds at
// 2^-48 of the date's sum (the sums are the curve's whole stochastic part,
// ~1e-2: ~1e-15 of the curve, random-walk-like over the run).  Entry (row
// b stride + s, slot B - j) holds three float4 {R_jk hi, CR_jk hi, R_jk lo,
// CR_jk lo} at lag (j - b) stride - 1 - s; rows are W.row slots wide.
//
// Windows, as the decomposition's response form (hjm_eresp.cu): the NS
// register slots hold the dates of one window [lo, hi] (dates
// 2 .. hi from max(lo, 2), slot r for date hi - r); a run with more dates is
// priced in launches over windows, the latest first, each re-running the
// normals from the first evolved step to date hi and passing the earlier
// windows its cash flows' sum and CVA share per path (carry).
struct VrespWindow {
    int lo, hi;  // the window's dates
    int row;     // slots per table row (global slot numbering, slot B - j for date j)
};

// NS register slots: 16 (128 registers, 8 CTAs per SM; windows of 16 dates,
// 6-7% faster than 24 slots at 6 CTAs per SM for 20 to 60 dates) or 24 (one
// launch for up to 24 dates: hjm_run_static, which has no carry).
template <int NT, bool EXT, int NS>
__global__ void __launch_bounds__(kFp64Cta, NS <= 16 ? 8 : 6)
    path_kernel_fp64_vresp(const __grid_constant__ PathParams<double> P, const VrespWindow W,
                           const float4* __restrict__ vresp, const double* __restrict__ ext,
                           double* __restrict__ partials, double* __restrict__ estore, double* __restrict__ carry)
{
    constexpr int kCta = kFp64Cta;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const int lo = W.lo, hi = W.hi;
    double* cf_s = reinterpret_cast<double*>(smem);  // [hi - lo + 3][kCta]: date i's cash flow in row i - lo + 1
    double* red_s = cf_s + (size_t)(hi - lo + 3) * kCta;

    const int64_t cta_base = (int64_t)blockIdx.x * kCta;
    const int64_t lp = cta_base + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;

    // {h at tenor j, its running sum} as hi + lo pairs, slot hi - j
    float2 A[NS], Al[NS];
#pragma unroll
    for (int r = 0; r < NS; ++r) A[r] = Al[r] = make_float2(0.0f, 0.0f);
    const int roff = B - hi;  // global slot of slot 0
    const int first = lo > 2 ? lo : 2;

    auto price = [&](int i) {
        double h = 0.0, hs = 0.0;
        if (i >= 2) {
            const float2 a = select_reg<NS, float2>(A, hi - i), l = select_reg<NS, float2>(Al, hi - i);
            h = widen_f32(a.x) + widen_f32(l.x);
            hs = widen_f32(a.y) + widen_f32(l.y);
        }
        const double x = P.psamp[i] + h;
        const double D = exp(-(P.psum[i] + hs) * P.dt);
        const double Lb = P.m * (exp(x * P.inv_m) - 1.0);
        cf_s[(size_t)(i - lo + 1) * kCta + tid] = D * (P.payA[i] * Lb - P.payB[i]);
    };

    if (lo == 1) price(1);
    for (int b = 1; b < hi; ++b) {
        const float4* row = vresp + ((size_t)b * P.stride * W.row + roff) * 3;
        // the window's dates still to be sampled: max(b + 1, first) .. hi
        const int n_act = hi - (b + 1 > first ? b + 1 : first) + 1;
        for (int s = 0; s < P.stride; ++s) {
            const int n = b * P.stride + s;
            float ph[3], pl[3];  // the normals as hi + lo (lo = 0 for the generator's FP32 draws)
            if constexpr (EXT) {
                double d0, d1, d2;
                draw_phi<double, true>(ext, gpath, active ? lp : 0, P.n_paths, n, P.rk0, P.rk1, d0, d1, d2);
                split_f64(d0, ph[0], pl[0]);
                split_f64(d1, ph[1], pl[1]);
                split_f64(d2, ph[2], pl[2]);
            } else {
                draw_phi<float, false>(ext, gpath, lp, P.n_paths, n, P.rk0, P.rk1, ph[0], ph[1], ph[2]);
            }
            const float4* rr = row + (size_t)s * W.row * 3;
            resp_groups(n_act, [&](auto gc) {
                constexpr int G = decltype(gc)::value;
                if constexpr (4 * G < NS) {
                float4 q[4][3];
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int k = 0; k < kFactors; ++k) q[u][k] = __ldg(rr + (4 * G + u) * 3 + k);
#pragma unroll
                for (int u = 0; u < 4; ++u) {
#pragma unroll
                    for (int k = 0; k < kFactors; ++k) {
                        const float2 kh = make_float2(q[u][k].x, q[u][k].y), kl = make_float2(q[u][k].z, q[u][k].w);
                        const float2 w = make_float2(ph[k], ph[k]), nw = make_float2(-ph[k], -ph[k]);
                        if constexpr (EXT)
                            df_acc(A[4 * G + u], Al[4 * G + u], kh, kl, w, make_float2(pl[k], pl[k]), nw);
                        else
                            df_acc_w(A[4 * G + u], Al[4 * G + u], kh, kl, w, nw);
                    }
                    df_renorm(A[4 * G + u], Al[4 * G + u]);
                }
                }
            });
        }
        if (b + 1 >= lo) price(b + 1);
    }
    window_epilogue<kCta>(P, lo, hi, cf_s, red_s, partials, estore, carry, cta_base, lp, active);
}

// Loadings of the three factors on the tenor grid (sqrt(dt) sigma_k, the
// predictor-corrector's N-projected ones), by value.
struct VolLoadings {
    double sv[kFactors][kMaxTenor];
};

// The table of path_kernel_fp64_vresp: R_jk(m) = (A^m S_k)[j] by m applications
// of the upwind step (Euler: backward difference at L, simulation_cpu.h:96-108)
// or of A2 (predictor-corrector: three-point stencil, Euler rows at L-1, L),
// and their running sums; the lag -> entry map of eresp_table_kernel.  One
// CTA of kMaxTenor threads, thread t holding tenor t of the three responses.
__global__ void __launch_bounds__(kMaxTenor)
    response_table_vol_kernel(int nt, double c, int stride, int B, int row, int pc,
                              const __grid_constant__ VolLoadings S, float4* __restrict__ vresp)
{
    __shared__ double v_s[kFactors][kMaxTenor];
    const int t = threadIdx.x;
    const int L = nt - 1;
    const int M = (B - 1) * stride - 1;
    const double a0 = 1.0 - c + 0.5 * c * c, a1 = c - c * c, a2 = 0.5 * c * c;
    double v[kFactors], cum[kFactors];
#pragma unroll
    for (int k = 0; k < kFactors; ++k) {
        v[k] = t < nt ? S.sv[k][t] : 0.0;
        cum[k] = 0.0;
    }
    for (int m = 0; m <= M; ++m) {
#pragma unroll
        for (int k = 0; k < kFactors; ++k) cum[k] += v[k];
        if (t >= 2 && t <= B) {
            const int q = m / stride + 1;
            const int b = t - q;
            if (b >= 1) {
                float4* e = vresp + (((size_t)b * stride + (size_t)(q * stride - 1 - m)) * row + (B - t)) * 3;
#pragma unroll
                for (int k = 0; k < kFactors; ++k) {
                    const float vh = __double2float_rn(v[k]), ch = __double2float_rn(cum[k]);
                    e[k] = make_float4(vh, ch, __double2float_rn(v[k] - (double)vh),
                                       __double2float_rn(cum[k] - (double)ch));
                }
            }
        }
#pragma unroll
        for (int k = 0; k < kFactors; ++k) v_s[k][t] = v[k];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < kFactors; ++k) {
            if (!pc) {
                if (t < L)
                    v[k] += c * (v_s[k][t + 1] - v[k]);
                else if (t == L)
                    v[k] += c * (v[k] - v_s[k][L - 1]);
            } else {
                if (t < L - 1)
                    v[k] = a0 * v[k] + a1 * v_s[k][t + 1] + a2 * v_s[k][t + 2];
                else if (t == L - 1)
                    v[k] += c * (v_s[k][L] - v[k]);
                else if (t == L)
                    v[k] += c * (v[k] - v_s[k][L - 1]);
            }
        }
        __syncthreads();
    }
}

// Mixed precision with packed FP32x2 arithmetic.  The curve of one path is held
// as H = ceil(NT/2) float2 pairs, pair p = {h[p], h[p+H]}: the upwind neighbour
// h[t+1] of every tenor lies in the same component of pair p+1, so each packed
// FMA (__ffma2_rn) advances two tenors: with the growth scaling of PathParams
// the polynomial form's step is one packed FMA per pair, the table form's four.
// Only the seam pair (p = H-1, whose .x neighbour is pair 0's .y), the pair
// holding the last tenor (backward difference) and the padding tenor of an odd
// grid take scalar fix-ups.
// ---------------------------------------------------------------------------
// Mixed-precision discount sums: FP32 block sums by the same recovery as the
// FP64 kernel, but anchored at tenor 1 and run upwards,
//     H[t+1] = H[t] - (sum_k sv[k][t] Phi_k - (A d)[t]) / c,   t = 1 .. B-1,
// so a block costs O(B) scalar FP32 operations and four additions per step
// (Phi_k and H[1]) instead of an addition per tenor per step; the FP32 block
// sums are then folded into FP64 per tenor.  The recovered sums differ from
// step-by-step FP32 accumulation by ~1e-6 relative (the FP32 rounding of the
// Euler steps divided by c), far inside the mixed-precision tolerance.
//
// Shared memory per thread: acc (B+1) FP64 discount sums, whose slot i holds
// date i's cash flow once tenor i is sampled; hs (B+2) FP32 curve at the block
// start, reused for the exposure tile at the end.
// CMP (polynomial factors, many dates): acc holds FP32 instead, the sums of the
// convected remainder only (its block sums in FP32, as folded into FP64
// otherwise; the remainder is a small fraction of the curve), and the FP64
// running sums of the scalar parts S, U, W stay in registers, so that the
// shared memory of a CTA (the occupancy limit with 60 dates) shrinks by a third.
// Occupancy: 512 threads per SM by the registers (<= 128 per thread; 112 with
// polynomial factors, 4 CTAs of 128).  Capped at 96 registers (5 CTAs, 20
// warps) the polynomial form does not spill but ran slower (20.8 ms against
// 20.5 at 4,194,304 paths); the compact sums' 64-thread CTAs are bounded by
// shared memory first (7 per SM for the netting set).
template <int NT, bool EXT, bool POLY, bool CMP, int C, bool CUB = false>
__global__ void __launch_bounds__(C, 512 / C)
    path_kernel_mixed(const __grid_constant__ MixedParams M, const double* __restrict__ ext,
                      double* __restrict__ partials, float* __restrict__ estore)
{
    static_assert(!CMP || POLY, "the compact sums need the polynomial parts");
    static_assert(!CUB || POLY, "the cubic part extends the polynomial form");
    using Acc = typename std::conditional<CMP, float, double>::type;
    const PathParams<float>& P = M.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const int rows = B + 1;
    constexpr size_t ka = sizeof(Acc);
    Acc* acc_s = reinterpret_cast<Acc*>(smem);                                // [B+1][C]
    float* hs_s = reinterpret_cast<float*>(smem + (size_t)rows * C * ka);  // [B+2][C]
    double* red_s = reinterpret_cast<double*>(
        smem + (((size_t)rows * C * ka + (size_t)(rows + 1) * C * 4 + 7) & ~(size_t)7));
    double zS = 0.0, zU = 0.0, zW = 0.0, zX = 0.0;  // CMP: FP64 running sums of the parts over the evolved steps

    const int64_t cta_base = (int64_t)blockIdx.x * C;
    const int64_t lp = cta_base + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;

    MixedPath<NT, POLY, CUB> x;
    x.reset();
    for (int i = 0; i < rows; ++i) acc_s[i * C + tid] = Acc(0);
    for (int t = 0; t <= B + 1; ++t) hs_s[t * C + tid] = 0.f;

    auto sample = [&](int i) {
        const double xv = P.psamp[i] + (double)x.value(P, i);
        double a = P.psum[i] + as_f64(acc_s[i * C + tid]);
        if constexpr (CMP) {
            const double ti = (double)P.tau[i];
            a += CUB ? fma(ti, fma(ti, fma(ti, zX, zW), zU), zS) : fma(ti, fma(ti, zW, zU), zS);
        }
        const float D = expf((float)(-a * P.dt));
        const float mm = (float)P.m;
        const float L = mm * expm1f((float)xv / mm);
        const float cf = D * ((float)P.payA[i] * L - (float)P.payB[i]);
        acc_s[i * C + tid] = (Acc)cf;  // cash flow of date i
    };

    sample(1);
    // normals drawn one step ahead, so that the generator's dependent chain
    // overlaps the curve update (the last step redraws itself, unused)
    const int n_last = B * P.stride - 1;
    const int64_t lpc = active ? lp : 0;
    float q0, q1, q2;
    draw_phi<float, EXT>(ext, gpath, lpc, P.n_paths, min(P.stride, n_last), P.rk0, P.rk1, q0, q1, q2);
    for (int b = 1; b < B; ++b) {
        BlockSums bs;
        bs.reset();
        x.begin_block(P, b);
#pragma unroll(POLY ? 2 : 1)  // ping-pong the normals drawn ahead instead of copying them
        for (int s = 0; s < P.stride; ++s) {
            const int n = b * P.stride + s;
            const float phi0 = q0, phi1 = q1, phi2 = q2;
            draw_phi<float, EXT>(ext, gpath, lpc, P.n_paths, min(n + 1, n_last), P.rk0, P.rk1, q0, q1, q2);
            x.step(M, phi0, phi1, phi2);
            bs.add(x, phi0, phi1, phi2);
        }
        // block sums of tenors 2 .. B; fold (b, B] into FP64 (CMP: the
        // remainder's in FP32, the parts' into their FP64 running sums)
        if constexpr (CMP) {
            recover_sums_up<NT>(x.h, hs_s, tid, C, P, x.g, 0.f, 0.f, 0.f, bs.H1, B, [&](int t, float Ht) {
                if (t > b) acc_s[t * C + tid] += Ht;
            });
            zS += as_f64(bs.sS);
            zU += as_f64(bs.sU);
            zW += as_f64(bs.sW);
            if constexpr (CUB) zX += as_f64(bs.sX);
        } else {
            block_sums_up<NT, POLY>(x, hs_s, tid, C, P, bs, B, [&](int t, float Ht) {
                if (t > b) acc_s[t * C + tid] += as_f64(Ht);
            });
        }
        // the block-end curve (POLY: its convected part) is the next block's start
#pragma unroll
        for (int t = 1; t < NT; ++t)
            if (t <= B + 1) hs_s[t * C + tid] = x.rem(t);
        sample(b + 1);
    }

    mixed_epilogue<Acc, C>(P, acc_s, hs_s, red_s, partials, estore, cta_base, active);
}

__host__ __device__ inline size_t mixed_smem_bytes(int nt, int n_blocks, bool cmp = false, int cta = kCta)
{
    (void)nt;
    const size_t rows = (size_t)n_blocks + 1;
    const size_t head = rows * cta * (cmp ? 4 : 8) + (rows + 1) * cta * 4;
    return ((head + 7) & ~(size_t)7) + 2 * (cta / 32) * 8;
}

// The compact sums when the FP64 ones would hold a CTA's shared memory above a
// quarter of the SM's (fewer than the 4 CTAs the registers allow)
inline bool mixed_compact(int nt, int n_blocks, bool poly)
{
    return poly && mixed_smem_bytes(nt, n_blocks, false) > (size_t)228 * 1024 / 4;
}

// Paths per CTA of the mixed kernel.  With the compact sums shared memory
// bounds the occupancy (~0.5 KB per path with 60 dates), and 64-thread CTAs
// pack an SM more finely: 7 of them (14 warps) where 3 of 128 threads fit
// (12 warps) for the 61-tenor netting set (36.5 ms from 37.1); a 25y swap on
// 51 tenors keeps 16 warps either way.  Otherwise the registers bound it,
// whatever the CTA size.
// The table step keeps FP64 sums per tenor (no compact form without the
// parts), so with many dates its shared memory binds the same way (25y on 51
// tenors: 79 KB per CTA of 128, 2 per SM; 5 of 64, 10 warps instead of 8).
constexpr int kMixedCompactCta = 64;
inline int mixed_cta(int nt, int n_blocks, bool poly)
{
    if (mixed_compact(nt, n_blocks, poly)) return kMixedCompactCta;
    return mixed_smem_bytes(nt, n_blocks, false) > (size_t)228 * 1024 / 4 ? kMixedCompactCta : kCta;
}

void pack_mixed_params(int nt, const PathParams<float>& P, MixedParams& M)
{
    std::memset(&M, 0, sizeof(M));
    M.P = P;
    const int H = (nt + 1) / 2;
    for (int k = 0; k < kFactors; ++k)
        for (int p = 0; p < H; ++p) {
            M.svp[k][p].x = P.sv[k][p];
            M.svp[k][p].y = (H + p < nt) ? P.sv[k][H + p] : 0.0f;
        }
    M.rp = make_float2(P.rr, P.rr);
    for (int k = 0; k < kFactors; ++k)
        for (int d = 0; d < 3; ++d) M.svcf[k][d] = (float)P.svc[k][d];
    M.k1f = (float)P.k1;
    M.k2f = (float)P.k2;
}

// ---------------------------------------------------------------------------
// Deterministic column sums of the CTA partials (Neumaier-compensated FP64):
// one CTA per column, fixed assignment of rows to threads, fixed tree order.
// Replaces the cuBLAS gemv with a ones vector (simulation_gpu.cu:889-933) and
// the host vAdd/saxpy (simulation_gpu.cu:941-951, 1157-1179).
// ---------------------------------------------------------------------------
constexpr int kReduceThreads = 256;

__device__ __forceinline__ void neumaier_add(double& s, double& comp, double x)
{
    const double t = s + x;
    comp += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
}

__global__ void __launch_bounds__(kReduceThreads)
    reduce_columns(const double* __restrict__ partials, int64_t n_rows, int R, double* __restrict__ sums)
{
    __shared__ double ss[kReduceThreads], cs[kReduceThreads];
    const int col = blockIdx.x;
    double s = 0.0, comp = 0.0;
    for (int64_t r = threadIdx.x; r < n_rows; r += kReduceThreads) neumaier_add(s, comp, partials[(size_t)r * R + col]);
    ss[threadIdx.x] = s;
    cs[threadIdx.x] = comp;
    __syncthreads();
    for (int w = kReduceThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            double a = ss[threadIdx.x], ca = cs[threadIdx.x] + cs[threadIdx.x + w];
            neumaier_add(a, ca, ss[threadIdx.x + w]);
            ss[threadIdx.x] = a;
            cs[threadIdx.x] = ca;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[col] = ss[0] + cs[0];
}

// EE, CVA, its standard error and dCVA/dhazard from the column sums.
__global__ void finalize_results(const double* __restrict__ sums, FinalParams F, double* __restrict__ result)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int B = F.n_blocks;
    const double inv_n = 1.0 / (double)F.n_paths;
    double cva = 0.0, dcva = 0.0;
    for (int j = 0; j < kMaxTenor; ++j) {
        const double ee = (j <= B) ? sums[j] * inv_n : 0.0;
        result[kResEE + j] = ee;
        cva += F.cvaw[j] * ee;
        dcva += F.dcvaw[j] * ee;
    }
    const double s1 = sums[B + 1], s2 = sums[B + 2];
    const double n = (double)F.n_paths;
    const double var = (n > 1.0) ? fmax((s2 - s1 * s1 / n) / (n - 1.0), 0.0) : 0.0;
    result[kResCVA] = cva;
    result[kResCVAStderr] = sqrt(var / n);
    result[kResDCVADHazard] = dcva;
    result[kResCVAPathMean] = s1 * inv_n;
}

// ---------------------------------------------------------------------------
// PFE: exact k-th smallest exposure of every date column by most-significant-
// digit radix selection on the IEEE bit patterns (exposures are >= +0, so the
// unsigned order of the bits is the numeric order).  11-bit digits; each pass
// histograms the candidates that match the prefix found so far.  Once a
// date's candidates number at most kPfeCap (two digits in, for a continuous
// distribution: 1/2048 of an octave), one more pass copies them to a buffer
// and one CTA ranks them in shared memory; the date's later passes exit at
// once.  A date whose candidates stay many (ties: e.g. most exposures zero)
// finishes by the global passes alone.  Three reads of the store instead of
// eight (FP64) or four (FP32) with 8-bit digits.
// ---------------------------------------------------------------------------
constexpr int kPfeDigit = 11;
constexpr int kPfeBins = 1 << kPfeDigit;

template <typename K>
__global__ void pfe_hist(const K* __restrict__ keys, int64_t ld, int64_t n, const SelState* __restrict__ st,
                         uint32_t* __restrict__ hist, int shift, int bits)
{
    __shared__ uint32_t h[kPfeBins];
    const int date = blockIdx.y;
    if (st[date].stage != 0) return;  // compacted: ranked in shared memory
    const int nb = 1 << bits;
    for (int i = threadIdx.x; i < nb; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const uint64_t prefix = st[date].prefix, mask = st[date].mask;
    const K* col = keys + (size_t)date * (size_t)ld;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        bool take = false;
        uint32_t digit = 0;
        if (i < n) {
            const uint64_t k = (uint64_t)col[i];
            take = (k & mask) == prefix;
            digit = (uint32_t)(k >> shift) & (uint32_t)(nb - 1);
        }
        // warp-aggregated increments: one atomic per distinct digit per warp
        const uint32_t active = __ballot_sync(0xffffffffu, take);
        if (take) {
            const uint32_t peers = __match_any_sync(active, digit);
            if ((threadIdx.x & 31) == (__ffs(peers) - 1)) atomicAdd(&h[digit], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < nb; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[(size_t)date * kPfeBins + i], h[i]);
}

// One CTA per date (256 threads): the digit whose cumulative count passes k,
// by a block-wide prefix sum over the bins (8 per thread); the histogram is
// cleared for the next pass.  A date left with at most kPfeCap candidates is
// marked for compaction (stage 1).
__global__ void __launch_bounds__(256) pfe_scan(SelState* __restrict__ st, uint32_t* __restrict__ hist, int shift,
                                                int bits)
{
    __shared__ uint32_t wsum[8];
    __shared__ int found;
    const int date = blockIdx.x;
    if (st[date].stage != 0) return;
    const int nb = 1 << bits;
    const int per = (nb + 255) / 256;  // bins per thread (8 at 11 bits)
    uint32_t* hd = hist + (size_t)date * kPfeBins;
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    uint32_t mine = 0;
    for (int b = 0; b < per; ++b) {
        const int bin = t * per + b;
        if (bin < nb) mine += hd[bin];
    }
    // exclusive prefix of the threads' sums
    uint32_t incl = mine;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[warp] = incl;
    if (t == 0) found = 0;
    __syncthreads();
    uint32_t before = incl - mine;
    for (int w = 0; w < warp; ++w) before += wsum[w];
    const uint64_t k = st[date].k;
    if ((uint64_t)before <= k && k < (uint64_t)before + mine) {
        uint64_t r = k - before;
        int d = t * per;
        for (;; ++d) {
            const uint32_t c = hd[d];
            if (r < c) break;
            r -= c;
        }
        const uint32_t cnt = hd[d];
        st[date].prefix |= (uint64_t)d << shift;
        st[date].mask |= (uint64_t)(nb - 1) << shift;
        st[date].k = r;
        st[date].count = cnt;
        if (cnt <= (uint32_t)kPfeCap && shift > 0) st[date].stage = 1;
        found = 1;
    }
    __syncthreads();
    for (int b = 0; b < per; ++b) {
        const int bin = t * per + b;
        if (bin < nb) hd[bin] = 0;
    }
}

// Copies the candidates of the dates marked for compaction (stage 1) to their
// buffers, warp-aggregated appends.
template <typename K>
__global__ void pfe_compact(const K* __restrict__ keys, int64_t ld, int64_t n, const SelState* __restrict__ st,
                            uint64_t* __restrict__ buf, uint32_t* __restrict__ cnt)
{
    const int date = blockIdx.y;
    if (st[date].stage != 1) return;
    const uint64_t prefix = st[date].prefix, mask = st[date].mask;
    const K* col = keys + (size_t)date * (size_t)ld;
    uint64_t* out = buf + (size_t)date * kPfeCap;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    const int lane = threadIdx.x & 31;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        uint64_t k = 0;
        bool take = false;
        if (i < n) {
            k = (uint64_t)col[i];
            take = (k & mask) == prefix;
        }
        const uint32_t ballot = __ballot_sync(0xffffffffu, take);
        if (ballot) {
            uint32_t at = 0;
            if (lane == __ffs(ballot) - 1) at = atomicAdd(&cnt[date], (uint32_t)__popc(ballot));
            at = __shfl_sync(0xffffffffu, at, __ffs(ballot) - 1);
            if (take) {
                const uint32_t pos = at + __popc(ballot & ((1u << lane) - 1u));
                if (pos < (uint32_t)kPfeCap) out[pos] = k;  // (the scan counted them: at most kPfeCap)
            }
        }
    }
}

// One CTA per compacted date: the candidate of rank k (ties by buffer
// position, so exactly one has it) becomes the date's key; stage 2.
__global__ void __launch_bounds__(256) pfe_finish(SelState* __restrict__ st, const uint64_t* __restrict__ buf,
                                                  uint32_t* __restrict__ cnt)
{
    __shared__ uint64_t c_s[kPfeCap];
    const int date = blockIdx.x;
    if (st[date].stage != 1) return;
    const uint32_t m = min(cnt[date], (uint32_t)kPfeCap);
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) c_s[i] = buf[(size_t)date * kPfeCap + i];
    __syncthreads();
    const uint64_t k = st[date].k;
    for (uint32_t i = threadIdx.x; i < m; i += blockDim.x) {
        const uint64_t v = c_s[i];
        uint32_t rank = 0;
        for (uint32_t j = 0; j < m; ++j) {
            const uint64_t w = c_s[j];
            rank += (w < v) || (w == v && j < i);
        }
        if (rank == k) st[date].prefix = v;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        st[date].mask = ~0ull;
        st[date].k = 0;
        st[date].stage = 2;
        cnt[date] = 0;
    }
}

template <typename K>
__global__ void pfe_write(const SelState* __restrict__ st, int n_dates, double* __restrict__ result)
{
    const int j = threadIdx.x;
    if (j < kMaxTenor) {
        double v = 0.0;
        if (j < n_dates) {
            if (sizeof(K) == 8) {
                v = __longlong_as_double((long long)st[j].prefix);
            } else {
                v = (double)__uint_as_float((uint32_t)st[j].prefix);
            }
        }
        result[kResPFE + j] = v;
    }
}

__global__ void pfe_init(SelState* __restrict__ st, int n_dates, uint64_t k0)
{
    const int j = threadIdx.x;
    if (j < n_dates) {
        st[j].prefix = 0;
        st[j].mask = 0;
        st[j].k = k0;
        st[j].count = 0;
        st[j].stage = 0;
    }
}

// ---------------------------------------------------------------------------
// Diagnostics: the device's normals and raw Philox words; layout transposes.
// ---------------------------------------------------------------------------
__global__ void dump_normals_kernel(int64_t n_paths, uint64_t path_offset, int n_steps, uint32_t k0, uint32_t k1,
                                    double* __restrict__ out)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n_paths * (int64_t)n_steps) return;
    const int64_t p = idx / n_steps;
    const int n = (int)(idx % n_steps);
    const uint4 w = philox4x32_10(normals_counter(path_offset + (uint64_t)p, (uint32_t)n), k0, k1);
    float z0, z1, z2;
    normals3(w, z0, z1, z2);
    out[idx * 3 + 0] = (double)z0;
    out[idx * 3 + 1] = (double)z1;
    out[idx * 3 + 2] = (double)z2;
}

__global__ void philox_words_kernel(int64_t n_paths, uint64_t path_offset, uint32_t step, uint32_t k0, uint32_t k1,
                                    uint32_t* __restrict__ out)
{
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_paths) return;
    const uint4 w = philox4x32_10(normals_counter(path_offset + (uint64_t)p, step), k0, k1);
    out[p * 4 + 0] = w.x;
    out[p * 4 + 1] = w.y;
    out[p * 4 + 2] = w.z;
    out[p * 4 + 3] = w.w;
}

// [path][step][3] -> [step][3][path] so that the path kernel reads coalesced
__global__ void transpose_normals_kernel(const double* __restrict__ in, int64_t n_paths, int n_steps,
                                         double* __restrict__ out)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = n_paths * (int64_t)n_steps * 3;
    if (idx >= total) return;
    const int64_t p = idx % n_paths;
    const int64_t rest = idx / n_paths;  // = n * 3 + k
    out[idx] = in[(size_t)p * n_steps * 3 + (size_t)rest];
}

// [date][ld] of T -> [date][n_paths] of double
template <typename T>
__global__ void widen_exposures_kernel(const T* __restrict__ in, int64_t ld, int64_t n_paths, int n_dates,
                                       double* __restrict__ out)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n_paths * (int64_t)n_dates) return;
    const int64_t j = idx / n_paths, p = idx % n_paths;
    out[idx] = (double)in[(size_t)j * ld + p];
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <int NT, bool EXT, int FORM>
static cudaError_t launch_fp64_t(const PathParams<double>& P, const double* ext, double* partials, double* estore,
                                 cudaStream_t s)
{
    const size_t smem = path_smem_bytes(NT, P.n_blocks, false);
    auto k = path_kernel_fp64<NT, EXT, FORM>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (P.n_paths + kFp64Cta - 1) / kFp64Cta;
    k<<<(unsigned)grid, kFp64Cta, smem, s>>>(P, ext, partials, estore);
    return cudaGetLastError();
}

template <int NT>
static cudaError_t launch_fp64_nt(const PathParams<double>& P, bool poly, const double* ext, double* partials,
                                  double* estore, cudaStream_t s)
{
    const bool tri = poly && P.svc[0][1] == 0.0 && P.svc[0][2] == 0.0 && P.svc[1][2] == 0.0;
    if (ext) return tri    ? launch_fp64_t<NT, true, kFormPolyTri>(P, ext, partials, estore, s)
                    : poly ? launch_fp64_t<NT, true, kFormPoly>(P, ext, partials, estore, s)
                           : launch_fp64_t<NT, true, kFormTable>(P, ext, partials, estore, s);
    return tri    ? launch_fp64_t<NT, false, kFormPolyTri>(P, ext, partials, estore, s)
           : poly ? launch_fp64_t<NT, false, kFormPoly>(P, ext, partials, estore, s)
                  : launch_fp64_t<NT, false, kFormTable>(P, ext, partials, estore, s);
}

cudaError_t launch_path_fp64(int nt, const PathParams<double>& P, bool poly, const double* ext, double* partials,
                             double* estore, cudaStream_t s)
{
    if (nt == 51) return launch_fp64_nt<51>(P, poly, ext, partials, estore, s);
    if (nt == 61) return launch_fp64_nt<61>(P, poly, ext, partials, estore, s);
    return cudaErrorInvalidValue;
}

template <int NT, bool EXT, int NS>
static cudaError_t launch_fp64_vresp_t(const PathParams<double>& P, const VrespWindow& W, const float4* vresp,
                                       const double* ext, double* partials, double* estore, double* carry,
                                       cudaStream_t s)
{
    // cf_s [hi - lo + 3][kCta] (the epilogue's exposures alias it one row up), red_s
    const size_t smem = ((size_t)(W.hi - W.lo + 3) * kFp64Cta + 2 * (kFp64Cta / 32)) * 8;
    auto k = path_kernel_fp64_vresp<NT, EXT, NS>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (P.n_paths + kFp64Cta - 1) / kFp64Cta;
    k<<<(unsigned)grid, kFp64Cta, smem, s>>>(P, W, vresp, ext, partials, estore, carry);
    return cudaGetLastError();
}

template <int NS>
static cudaError_t launch_fp64_vresp_ns(int nt, const PathParams<double>& P, const VrespWindow& W,
                                        const float4* vresp, const double* ext, double* partials, double* estore,
                                        double* carry, cudaStream_t s)
{
    if (nt == 51)
        return ext ? launch_fp64_vresp_t<51, true, NS>(P, W, vresp, ext, partials, estore, carry, s)
                   : launch_fp64_vresp_t<51, false, NS>(P, W, vresp, ext, partials, estore, carry, s);
    if (nt == 61)
        return ext ? launch_fp64_vresp_t<61, true, NS>(P, W, vresp, ext, partials, estore, carry, s)
                   : launch_fp64_vresp_t<61, false, NS>(P, W, vresp, ext, partials, estore, carry, s);
    return cudaErrorInvalidValue;
}

int vresp_windows(int n_blocks, int max_slots)
{
    return eresp_windows(n_blocks, 2, nullptr, nullptr, nullptr, max_slots);
}

cudaError_t launch_path_fp64_vresp(int nt, const PathParams<double>& P, const float4* vresp, const double* ext,
                                   double* partials, double* estore, double* carry, cudaStream_t s, int* launches,
                                   int max_slots)
{
    if (max_slots != 16 && max_slots != 24) return cudaErrorInvalidValue;
    int lo[kMaxTenor], hi[kMaxTenor];
    // every date is reached at once (the factors load every tenor): windows
    // of max_slots dates from date 2, the latest first
    const int nw = eresp_windows(P.n_blocks, 2, lo, hi, nullptr, max_slots);
    if (!vresp || (nw > 1 && !carry)) return cudaErrorInvalidValue;
    if (launches) *launches = 0;
    for (int w = 0; w < nw; ++w) {
        const VrespWindow W{lo[w], hi[w], vresp_row(P.n_blocks)};
        const cudaError_t e = max_slots == 16
                                  ? launch_fp64_vresp_ns<16>(nt, P, W, vresp, ext, partials, estore, carry, s)
                                  : launch_fp64_vresp_ns<24>(nt, P, W, vresp, ext, partials, estore, carry, s);
        if (e != cudaSuccess) return e;
        if (launches) ++*launches;
    }
    return cudaSuccess;
}

// Slots per row of the volatility-table response table: every date 2 .. B in
// its global slot B - j, and the last group of four a window reads (up to
// slot B + 1) within the row.
int vresp_row(int n_blocks) { return n_blocks + 2 <= kRespRow ? kRespRow : (n_blocks + 2 + 3) / 4 * 4; }

size_t response_table_vol_elems(int stride, int n_blocks)
{
    return (size_t)n_blocks * stride * vresp_row(n_blocks) * 3;
}

cudaError_t launch_response_table_vol(int nt, double c, int stride, int n_blocks, bool pc, const double* sv,
                                      float4* vresp, cudaStream_t s)
{
    if (nt < 3 || nt > kMaxTenor || n_blocks >= nt || stride < 1) return cudaErrorInvalidValue;
    VolLoadings S;
    std::memset(&S, 0, sizeof(S));
    for (int k = 0; k < kFactors; ++k)
        for (int t = 0; t < nt; ++t) S.sv[k][t] = sv[k * kMaxTenor + t];
    response_table_vol_kernel<<<1, kMaxTenor, 0, s>>>(nt, c, stride, n_blocks, vresp_row(n_blocks), pc ? 1 : 0, S,
                                                      vresp);
    return cudaGetLastError();
}

int response_max_dates() { return kRespDates; }

template <int NT, bool EXT, bool POLY, bool CUB = false>
static cudaError_t launch_mixed_t(const MixedParams& M, const double* ext, double* partials, float* estore,
                                  cudaStream_t s)
{
    const bool cmp = mixed_compact(NT, M.P.n_blocks, POLY);
    const int cta = mixed_cta(NT, M.P.n_blocks, POLY);
    const size_t smem = mixed_smem_bytes(NT, M.P.n_blocks, cmp, cta);
    auto k = path_kernel_mixed<NT, EXT, POLY, false, kCta, CUB>;
    if constexpr (POLY) {
        if (cmp) k = path_kernel_mixed<NT, EXT, true, true, kMixedCompactCta, CUB>;
    } else {
        if (cta == kMixedCompactCta) k = path_kernel_mixed<NT, EXT, false, false, kMixedCompactCta>;
    }
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (M.P.n_paths + cta - 1) / cta;
    k<<<(unsigned)grid, cta, smem, s>>>(M, ext, partials, estore);
    return cudaGetLastError();
}

template <int NT>
static cudaError_t launch_mixed_nt(const MixedParams& M, bool poly, bool cub, const double* ext, double* partials,
                                   float* estore, cudaStream_t s)
{
    if (cub) return ext ? launch_mixed_t<NT, true, true, true>(M, ext, partials, estore, s)
                        : launch_mixed_t<NT, false, true, true>(M, ext, partials, estore, s);
    if (ext) return poly ? launch_mixed_t<NT, true, true>(M, ext, partials, estore, s)
                         : launch_mixed_t<NT, true, false>(M, ext, partials, estore, s);
    return poly ? launch_mixed_t<NT, false, true>(M, ext, partials, estore, s)
                : launch_mixed_t<NT, false, false>(M, ext, partials, estore, s);
}

cudaError_t launch_path_mixed(int nt, const MixedParams& M, bool poly, const double* ext, double* partials,
                              float* estore, cudaStream_t s, bool cub)
{
    if (nt == 51) return launch_mixed_nt<51>(M, poly || cub, cub, ext, partials, estore, s);
    if (nt == 61) return launch_mixed_nt<61>(M, poly || cub, cub, ext, partials, estore, s);
    return cudaErrorInvalidValue;
}

bool path_tenor_supported(int nt) { return nt == 51 || nt == 61; }

size_t path_smem(int nt, int n_blocks, bool mixed)
{
    return mixed ? mixed_smem_bytes(nt, n_blocks) : path_smem_bytes(nt, n_blocks, false);  // the larger form
}

int path_cta(bool mixed, int nt, int n_blocks, bool poly)
{
    return mixed ? mixed_cta(nt, n_blocks, poly) : kFp64Cta;
}

cudaError_t launch_reduce(const double* partials, int64_t n_rows, int R, double* sums, const FinalParams& F,
                          double* result, cudaStream_t s)
{
    reduce_columns<<<R, kReduceThreads, 0, s>>>(partials, n_rows, R, sums);
    finalize_results<<<1, 32, 0, s>>>(sums, F, result);
    return cudaGetLastError();
}

size_t pfe_scratch_bytes()
{
    return sizeof(uint32_t) * ((size_t)kPfeBins * kMaxTenor + kMaxTenor) + sizeof(uint64_t) * (size_t)kPfeCap * kMaxTenor;
}

cudaError_t launch_pfe(const void* estore, bool fp64_keys, int64_t ld, int64_t n_paths, int n_dates, uint64_t k0,
                       SelState* st, void* scratch, double* result, int n_sms, cudaStream_t s)
{
    uint32_t* hist = (uint32_t*)scratch;
    uint32_t* cnt = hist + (size_t)kPfeBins * kMaxTenor;
    uint64_t* buf = (uint64_t*)(cnt + kMaxTenor);  // 8-byte aligned: kPfeBins * kMaxTenor + kMaxTenor is even
    pfe_init<<<1, kMaxTenor, 0, s>>>(st, n_dates, k0);
    cudaError_t e = cudaMemsetAsync(scratch, 0, sizeof(uint32_t) * ((size_t)kPfeBins * kMaxTenor + kMaxTenor), s);
    if (e != cudaSuccess) return e;
    int64_t gx = (n_paths + 1023) / 1024;
    const int64_t cap = (int64_t)n_sms * 8;
    if (gx > cap) gx = cap;
    if (gx < 1) gx = 1;
    const dim3 grid((unsigned)gx, (unsigned)n_dates);
    const int total = fp64_keys ? 64 : 32;
    for (int top = total; top > 0; top -= kPfeDigit) {
        const int bits = top < kPfeDigit ? top : kPfeDigit;
        const int shift = top - bits;
        if (fp64_keys) {
            pfe_hist<uint64_t><<<grid, 256, 0, s>>>((const uint64_t*)estore, ld, n_paths, st, hist, shift, bits);
        } else {
            pfe_hist<uint32_t><<<grid, 256, 0, s>>>((const uint32_t*)estore, ld, n_paths, st, hist, shift, bits);
        }
        pfe_scan<<<n_dates, 256, 0, s>>>(st, hist, shift, bits);
        if (shift == 0) break;
        if (fp64_keys)
            pfe_compact<uint64_t><<<grid, 256, 0, s>>>((const uint64_t*)estore, ld, n_paths, st, buf, cnt);
        else
            pfe_compact<uint32_t><<<grid, 256, 0, s>>>((const uint32_t*)estore, ld, n_paths, st, buf, cnt);
        pfe_finish<<<n_dates, 256, 0, s>>>(st, buf, cnt);
    }
    if (fp64_keys)
        pfe_write<uint64_t><<<1, kMaxTenor, 0, s>>>(st, n_dates, result);
    else
        pfe_write<uint32_t><<<1, kMaxTenor, 0, s>>>(st, n_dates, result);
    return cudaGetLastError();
}

cudaError_t launch_dump_normals(int64_t n_paths, uint64_t path_offset, int n_steps, uint32_t k0, uint32_t k1,
                                double* out, cudaStream_t s)
{
    const int64_t total = n_paths * (int64_t)n_steps;
    dump_normals_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n_paths, path_offset, n_steps, k0, k1, out);
    return cudaGetLastError();
}

cudaError_t launch_philox_words(int64_t n_paths, uint64_t path_offset, uint32_t step, uint32_t k0, uint32_t k1,
                                uint32_t* out, cudaStream_t s)
{
    philox_words_kernel<<<(unsigned)((n_paths + 255) / 256), 256, 0, s>>>(n_paths, path_offset, step, k0, k1, out);
    return cudaGetLastError();
}

cudaError_t launch_transpose_normals(const double* in, int64_t n_paths, int n_steps, double* out, cudaStream_t s)
{
    const int64_t total = n_paths * (int64_t)n_steps * 3;
    transpose_normals_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(in, n_paths, n_steps, out);
    return cudaGetLastError();
}

cudaError_t launch_widen_exposures(const void* in, bool fp64, int64_t ld, int64_t n_paths, int n_dates, double* out,
                                   cudaStream_t s)
{
    const int64_t total = n_paths * (int64_t)n_dates;
    const unsigned g = (unsigned)((total + 255) / 256);
    if (fp64)
        widen_exposures_kernel<double><<<g, 256, 0, s>>>((const double*)in, ld, n_paths, n_dates, out);
    else
        widen_exposures_kernel<float><<<g, 256, 0, s>>>((const float*)in, ld, n_paths, n_dates, out);
    return cudaGetLastError();
}

}  // namespace hjm
