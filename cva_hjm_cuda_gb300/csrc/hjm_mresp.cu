// hjm_mresp.cu -- the response form of the mixed-precision step (Euler and predictor-corrector).
//
// With polynomial volatility factors the stochastic curve splits as
//     h = S + U t + W t^2 (+ X t^3) + hc,
// the parts advancing as scalars (hjm_pairs.cuh, MixedPath) and the remainder
// hc, driven only at the last tenor by kappa w per step (kappa = -2 c dtau^2,
// w = W + 3 (T_L - tau0) X before the step), convected by the upwind step
// (backward difference at the last tenor, simulation_cpu.h:96-108).  The
// pricing of date j reads hc only at tenor j at its sampling step K_j = j
// stride - 1, with its running sum for the discount, so per date still to be
// sampled the kernel keeps those two numbers and adds per step
//     {kappa G_j(lag), kappa CG_j(lag)} w,   lag = K_j - n,
// G_j(m) = (A^m e_L)[j] and CG_j its running sum (the FP64 response form's
// algebra, hjm_eresp.cu, here in FP32 sums).  The convected form moves every
// tenor of hc per step (one packed FMA per two tenors, 26 at 51 tenors); the
// responses reach only the dates near the last tenor: on the 10y swap (20
// dates on 51 tenors, c = 0.02) no response of dates 2 to 12 ever reaches
// 2^-30 |kappa|, so eight slots (four packed FMAs per step) carry the
// remainder of every date whose response counts.
//
// Selection: the host counts, in FP64 (mresp_slots), the slots whose dates
// have a response that counts (a term of at least 2^-30
// |kappa|, or of its running sum at least 2^-30 |kappa| K_j: the dropped
// dates' remainders sum to ~1e-8 |kappa| max|w| per unit, far inside FP32's
// resolution of the curve); runs whose counting dates fit 8 or 16 slots take
// this kernel, the others (the 25y and 30y runs: 38 and 44 slots) the
// convected form.
//
// The predictor-corrector step runs the same kernel: its parts advance by
// the same update with the N-projected loadings and (c + c^2) dtau^2, and its
// remainder, driven at L - 1 and L by the old and the new W, has per old W
// the responses H(l) = w0 G1(l) + w1 G2(l) + w2 G2(l + 1) of the three-point
// step (mresp_table_pc_kernel); a run whose last date samples the last tenor
// (its own step's new W enters there with no lag) convects.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "hjm_epilogue.cuh"
#include "hjm_kernels.h"

namespace hjm {

namespace {

// CTAs per SM of the response kernel with ns slots: the registers' bound
// (8 slots in 80 registers, 6 CTAs; 16 spill below 128 registers, 4 CTAs)
constexpr int mresp_min_ctas(int ns) { return ns <= 8 ? 6 : 4; }

}  // namespace

// EXT: external normals; CUB: the cubic part X (P.tau holds T - tau0); NS:
// date slots (8 or 16), slot r holding date B - r.  resp: rows b stride + s of
// NS / 2 float4, each two {kappa G, kappa CG} pairs (mresp_table_kernel).
template <bool EXT, bool CUB, int NS>
__global__ void __launch_bounds__(kCta, mresp_min_ctas(NS))
    path_kernel_mixed_resp(const __grid_constant__ MixedParams M, const float4* __restrict__ resp,
                           const double* __restrict__ ext, double* __restrict__ partials,
                           float* __restrict__ estore)
{
    constexpr int C = kCta;
    const PathParams<float>& P = M.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    // cash flows of dates 1..B in rows 1..B (FP32, as the kernel prices
    // them); the epilogue's exposures alias them one row up (row j + 1 holds
    // exposure j once cash flow j + 1 is read)
    float* cf_s = reinterpret_cast<float*>(smem);                                 // [B + 2][C]
    double* red_s = reinterpret_cast<double*>(smem + (size_t)(B + 2) * C * sizeof(float));

    const int64_t cta_base = (int64_t)blockIdx.x * C;
    const int64_t lp = cta_base + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;

    float2 A[NS];  // {hc at date j's tenor, its running sum}, slot B - j
#pragma unroll
    for (int r = 0; r < NS; ++r) A[r] = make_float2(0.f, 0.f);
    float S = 0.f, U = 0.f, W = 0.f, X = 0.f;
    double zS = 0.0, zU = 0.0, zW = 0.0, zX = 0.0;  // FP64 running sums of the parts over the evolved steps

    // price date i from the remainder's value and running sum at its tenor
    auto price = [&](int i, float2 rc) {
        const float ti = P.tau[i];
        const float pv = CUB ? fmaf(ti, fmaf(ti, fmaf(ti, X, W), U), S) : fmaf(ti, fmaf(ti, W, U), S);
        const double xv = P.psamp[i] + (double)(rc.x + pv);
        const double td = (double)ti;
        const double zp = CUB ? fma(td, fma(td, fma(td, zX, zW), zU), zS) : fma(td, fma(td, zW, zU), zS);
        const double a = P.psum[i] + (double)rc.y + zp;
        const float D = expf((float)(-a * P.dt));
        const float mm = (float)P.m;
        const float L = mm * expm1f((float)xv / mm);
        cf_s[i * C + tid] = D * ((float)P.payA[i] * L - (float)P.payB[i]);
    };

    price(1, make_float2(0.f, 0.f));  // the first block holds the curve at spot
    // normals drawn one step ahead, so that the generator's dependent chain
    // overlaps the step's updates (the last step redraws itself, unused)
    const int n_last = B * P.stride - 1;
    const int64_t lpc = active ? lp : 0;
    float q0, q1, q2;
    draw_phi<float, EXT>(ext, gpath, lpc, P.n_paths, min(P.stride, n_last), P.rk0, P.rk1, q0, q1, q2);
    for (int b = 1; b < B; ++b) {
        float sS = 0.f, sU = 0.f, sW = 0.f, sX = 0.f;
        const float4* row = resp + (size_t)b * P.stride * (NS / 2);
        // unrolled by 5 (a divisor of 50 steps per block; the generator's
        // draws of five steps in flight): 15.65 ms at 4M paths on the 10y
        // swap, against 15.77 by 4 and 16.67 by 2; the cubic, 16-slot and
        // external-normals variants spill beyond 2
#pragma unroll((EXT || CUB || NS > 8) ? 2 : 5)
        for (int s = 0; s < P.stride; ++s) {
            const int n = b * P.stride + s;
            const float phi0 = q0, phi1 = q1, phi2 = q2;
            draw_phi<float, EXT>(ext, gpath, lpc, P.n_paths, min(n + 1, n_last), P.rk0, P.rk1, q0, q1, q2);
            // the remainder's source w before the step's update, into every slot
            const float w = CUB ? fmaf(M.src3f, X, W) : W;
            const float2 w2 = make_float2(w, w);
            const float4* rr = row + (size_t)s * (NS / 2);
#pragma unroll
            for (int u = 0; u < NS / 2; ++u) {
                const float4 e = __ldg(rr + u);
                A[2 * u] = __ffma2_rn(make_float2(e.x, e.y), w2, A[2 * u]);
                A[2 * u + 1] = __ffma2_rn(make_float2(e.z, e.w), w2, A[2 * u + 1]);
            }
            // the parts (MixedPath::step's polynomial update: old U, W, X on the right)
            float Sn = fmaf(M.svcf[0][0], phi0, fmaf(M.k2f, W, fmaf(M.k1f, U, S)));
            if constexpr (CUB) Sn = fmaf(M.k3f, X, Sn);
            Sn = fmaf(M.svcf[2][0], phi2, fmaf(M.svcf[1][0], phi1, Sn));
            float Un = fmaf(M.svcf[1][1], phi1, fmaf(M.svcf[0][1], phi0, fmaf(2.0f * M.k1f, W, U)));
            if constexpr (CUB) Un = fmaf(3.0f * M.k2f, X, Un);
            Un = fmaf(M.svcf[2][1], phi2, Un);
            float Wn = fmaf(M.svcf[2][2], phi2, fmaf(M.svcf[1][2], phi1, fmaf(M.svcf[0][2], phi0, W)));
            if constexpr (CUB) {
                Wn = fmaf(3.0f * M.k1f, X, Wn);
                X = fmaf(M.svcx[2], phi2, fmaf(M.svcx[1], phi1, fmaf(M.svcx[0], phi0, X)));
                sX += X;
            }
            S = Sn;
            U = Un;
            W = Wn;
            sS += S;
            sU += U;
            sW += W;
        }
        zS += (double)sS;
        zU += (double)sU;
        zW += (double)sW;
        if constexpr (CUB) zX += (double)sX;
        const int i = b + 1;
        const int r = B - i;  // (a slot beyond NS holds a date whose response never counts)
        price(i, r < NS ? select_reg<NS, float2>(A, r) : make_float2(0.f, 0.f));
    }
    mixed_epilogue<float, C>(P, cf_s, cf_s + C, red_s, partials, estore, cta_base, active);
}

// ---------------------------------------------------------------------------
// Host
// ---------------------------------------------------------------------------
size_t mresp_smem_bytes(int n_blocks) { return (size_t)(n_blocks + 2) * kCta * sizeof(float) + 2 * (kCta / 32) * 8; }

// The predictor-corrector's remainder sources per unit W: w0 W_old at L - 1,
// w1 W_old + w2 W_new at L (w0 = -c^2 dtau^2, w1 = -(c + c^2) dtau^2, w2 =
// -c dtau^2; their sum is the step's kappa).
static void pc_sources(double c, double dtau, double& w0, double& w1, double& w2)
{
    const double d2 = dtau * dtau;
    w0 = -c * c * d2;
    w1 = -(c + c * c) * d2;
    w2 = -c * d2;
}

int mresp_slots(int nt, double c, double dtau, int stride, int n_blocks, bool pc)
{
    const int B = n_blocks, L = nt - 1;
    if (nt < 3 || nt > kMaxTenor || B < 1 || B >= nt || stride < 1 || !(c > 0.0 && c < 1.0)) return 0;
    // (the predictor-corrector's date at the last tenor takes a lag -1 term
    // this kernel leaves out)
    if (pc && B == L) return 0;
    const double thr = std::ldexp(1.0, -30);
    const int M = (B - 1) * stride - 1;  // the longest lag read
    // Euler: G = A^m e_L.  Predictor-corrector: H(l) = w0 G1(l) + w1 G2(l) +
    // w2 G2(l + 1) per unit kappa, G1, G2 the three-point step's responses to
    // e_{L-1}, e_L (the tables' recursions, eresp_table_pc_kernel)
    double w0 = 0.0, w1 = 0.0, w2 = 0.0, kap = 1.0;
    if (pc) {
        pc_sources(c, dtau, w0, w1, w2);
        kap = std::fabs(w0 + w1 + w2);
    }
    const double a0 = 1.0 - c + 0.5 * c * c, a1 = c - c * c, a2 = 0.5 * c * c;
    double v[kMaxTenor] = {}, vn[kMaxTenor], cum[kMaxTenor] = {};   // Euler, or G2 for the predictor-corrector
    double u[kMaxTenor] = {}, un[kMaxTenor], cu[kMaxTenor] = {};    // G1
    double hp[kMaxTenor] = {}, chp[kMaxTenor] = {};                 // w0 G1 + w1 G2 at the previous lag
    v[L] = 1.0;
    if (pc) u[L - 1] = 1.0;
    int need = 0;
    for (int m = 0; m <= M + (pc ? 1 : 0); ++m) {
        for (int t = 0; t < nt; ++t) {
            cum[t] += v[t];
            cu[t] += u[t];
        }
        const int l = pc ? m - 1 : m;  // the lag this iteration completes
        if (l >= 0)
            for (int j = 2; j < B + 1 - need; ++j) {
                // date j reads lags up to K_j - stride = (j - 1) stride - 1
                if (l > (j - 1) * stride - 1) continue;
                const double h = pc ? (hp[j] + w2 * v[j]) / kap : v[j];
                const double ch = pc ? (chp[j] + w2 * cum[j]) / kap : cum[j];
                if (std::fabs(h) >= thr || std::fabs(ch) >= thr * (double)(j * stride)) need = B - j + 1;
            }
        if (pc) {
            for (int t = 0; t < nt; ++t) {
                hp[t] = w0 * u[t] + w1 * v[t];
                chp[t] = w0 * cu[t] + w1 * cum[t];
            }
            for (int t = 0; t < L - 1; ++t) {
                vn[t] = a0 * v[t] + a1 * v[t + 1] + a2 * v[t + 2];
                un[t] = a0 * u[t] + a1 * u[t + 1] + a2 * u[t + 2];
            }
            vn[L - 1] = v[L - 1] + c * (v[L] - v[L - 1]);
            un[L - 1] = u[L - 1] + c * (u[L] - u[L - 1]);
            vn[L] = v[L] + c * (v[L] - v[L - 1]);
            un[L] = u[L] + c * (u[L] - u[L - 1]);
            for (int t = 0; t < nt; ++t) u[t] = un[t];
        } else {
            for (int t = 0; t < L; ++t) vn[t] = v[t] + c * (v[t + 1] - v[t]);
            vn[L] = v[L] + c * (v[L] - v[L - 1]);
        }
        for (int t = 0; t < nt; ++t) v[t] = vn[t];
    }
    return need <= 8 ? 8 : (need <= 16 ? 16 : 0);
}

size_t mresp_table_elems(int stride, int n_blocks, int ns) { return (size_t)n_blocks * stride * (ns / 2); }

// The table: for date j = B - r (slot r < ns) at lag m <= (j - 1) stride - 1,
// row n = j stride - 1 - m (>= stride) holds {kappa G_j(m), kappa CG_j(m)} in
// float2 r of the row; the rest stays zero (cleared by the launcher).  FP64
// recursion, one CTA, thread t holding tenor t.
__global__ void __launch_bounds__(kMaxTenor)
    mresp_table_kernel(int nt, double c, int stride, int B, int ns, double kappa, float4* __restrict__ table)
{
    __shared__ double v_s[kMaxTenor];
    const int t = threadIdx.x;
    const int L = nt - 1;
    const int M = (B - 1) * stride - 1;
    const int r = B - t;
    const bool keep = t >= 2 && t <= B && r < ns;
    double v = (t == L) ? 1.0 : 0.0, cum = 0.0;
    float2* row2 = reinterpret_cast<float2*>(table);
    for (int m = 0; m <= M; ++m) {
        cum += v;
        if (keep && m <= (t - 1) * stride - 1) {
            const size_t n = (size_t)t * stride - 1 - (size_t)m;
            row2[n * ns + r] = make_float2((float)(kappa * v), (float)(kappa * cum));
        }
        v_s[t] = v;
        __syncthreads();
        if (t < L)
            v += c * (v_s[t + 1] - v);
        else if (t == L)
            v += c * (v - v_s[L - 1]);
        __syncthreads();
    }
}

// The predictor-corrector's table in the same layout: per old W at lag l,
// {H(l), CH(l)} with H(l) = w0 G1(l) + w1 G2(l) + w2 G2(l + 1) (W_new of one
// step is W_old of the next) and CH likewise from the running sums, the
// recursions of eresp_table_pc_kernel (hjm_eresp.cu) rounded to FP32.
__global__ void __launch_bounds__(kMaxTenor)
    mresp_table_pc_kernel(int nt, double c, int stride, int B, int ns, double w0, double w1, double w2,
                          float4* __restrict__ table)
{
    __shared__ double v_s[kMaxTenor + 2], u_s[kMaxTenor + 2];
    const int t = threadIdx.x;
    const int L = nt - 1;
    const int M = (B - 1) * stride - 1;
    const double a0 = 1.0 - c + 0.5 * c * c, a1 = c - c * c, a2 = 0.5 * c * c;
    const int r = B - t;
    const bool keep = t >= 2 && t <= B && r < ns;
    double g1 = (t == L - 1) ? 1.0 : 0.0, g2 = (t == L) ? 1.0 : 0.0;
    double cg1 = 0.0, cg2 = 0.0, hp = 0.0, chp = 0.0;
    float2* row2 = reinterpret_cast<float2*>(table);
    for (int m = 0; m <= M + 1; ++m) {
        cg1 += g1;
        cg2 += g2;
        const int l = m - 1;  // the lag this iteration completes
        if (keep && l >= 0 && l <= (t - 1) * stride - 1) {
            const size_t n = (size_t)t * stride - 1 - (size_t)l;
            row2[n * ns + r] = make_float2((float)(hp + w2 * g2), (float)(chp + w2 * cg2));
        }
        hp = w0 * g1 + w1 * g2;
        chp = w0 * cg1 + w1 * cg2;
        if (t < nt) {
            v_s[t] = g1;
            u_s[t] = g2;
        }
        __syncthreads();
        if (t < L - 1) {
            g1 = a0 * g1 + a1 * v_s[t + 1] + a2 * v_s[t + 2];
            g2 = a0 * g2 + a1 * u_s[t + 1] + a2 * u_s[t + 2];
        } else if (t == L - 1) {
            g1 += c * (v_s[L] - g1);
            g2 += c * (u_s[L] - g2);
        } else if (t == L) {
            g1 += c * (g1 - v_s[L - 1]);
            g2 += c * (g2 - u_s[L - 1]);
        }
        __syncthreads();
    }
}

cudaError_t launch_mresp_table(int nt, double c, double dtau, int stride, int n_blocks, int ns, bool pc,
                               float4* table, cudaStream_t s)
{
    if (nt < 3 || nt > kMaxTenor || n_blocks < 1 || n_blocks >= nt || stride < 1 || (ns != 8 && ns != 16))
        return cudaErrorInvalidValue;
    cudaError_t e = cudaMemsetAsync(table, 0, sizeof(float4) * mresp_table_elems(stride, n_blocks, ns), s);
    if (e != cudaSuccess) return e;
    if (pc) {
        double w0, w1, w2;
        pc_sources(c, dtau, w0, w1, w2);
        mresp_table_pc_kernel<<<1, kMaxTenor, 0, s>>>(nt, c, stride, n_blocks, ns, w0, w1, w2, table);
    } else {
        mresp_table_kernel<<<1, kMaxTenor, 0, s>>>(nt, c, stride, n_blocks, ns, -2.0 * c * dtau * dtau, table);
    }
    return cudaGetLastError();
}

namespace {

template <bool EXT, bool CUB>
cudaError_t launch_mresp_t(const MixedParams& M, int ns, const float4* table, const double* ext, double* partials,
                           float* estore, cudaStream_t s)
{
    auto k = ns == 8 ? path_kernel_mixed_resp<EXT, CUB, 8> : path_kernel_mixed_resp<EXT, CUB, 16>;
    const size_t smem = mresp_smem_bytes(M.P.n_blocks);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (M.P.n_paths + kCta - 1) / kCta;
    k<<<(unsigned)grid, kCta, smem, s>>>(M, table, ext, partials, estore);
    return cudaGetLastError();
}

}  // namespace

cudaError_t launch_path_mixed_resp(const MixedParams& M, int ns, bool cub, const float4* table, const double* ext,
                                   double* partials, float* estore, cudaStream_t s)
{
    if (ns != 8 && ns != 16) return cudaErrorInvalidValue;
    if (M.P.n_blocks < 1 || M.P.n_blocks >= kMaxTenor || M.P.stride < 1) return cudaErrorInvalidValue;
    if (ext) return cub ? launch_mresp_t<true, true>(M, ns, table, ext, partials, estore, s)
                        : launch_mresp_t<true, false>(M, ns, table, ext, partials, estore, s);
    return cub ? launch_mresp_t<false, true>(M, ns, table, ext, partials, estore, s)
               : launch_mresp_t<false, false>(M, ns, table, ext, partials, estore, s);
}

}  // namespace hjm
