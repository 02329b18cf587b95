// hjm_eresp.cu -- the FP64 response form of the Euler step: polynomial parts
// of degree <= 3, a residual volatility table, and runs of any number of
// dates in windows of at most kRespSlots.
//
// The stochastic curve h (f = p + h, p the deterministic curve) is split as
//     h = sum_d x_d t^d + hc,   t = T - tau0,
// the parts x_d advancing by x <- M x + B phi (hjm_resp.cuh states M and the
// moving frame), and the remainder hc by hc <- A hc + kappa w e_L + r phi,
// where A is the upwind step (backward difference at the last tenor,
// simulation_cpu.h:96-108), kappa w e_L the polynomial's error at L (kappa =
// -2 c dtau^2, w = x_2 + 3 (T_L - tau0) x_3 before the step), and r the
// residual loadings sqrt(dt) (sigma_k - poly_k) of a volatility table that
// is a cubic only to its printed precision (the reference's own PCA table,
// simulation_gpu_testing.cpp:47-63: factors 2 and 3 are cubics to 1.1e-7 of
// their scale).  The pricing reads hc only at date j's tenor at its sampling
// step, so per date still to be sampled the kernel keeps hc[j] and its
// running sum, adding per step
//     kappa G_j(lag) W            (double-FP32, the W terms: A, Al)
//   + sum_k R_jk(lag) phi_k        (FP32 into the low lanes Al: the residual)
// with G_j(m) = (A^m e_L)[j], R_jk(m) = (A^m r_k)[j] and their running sums
// (eresp_table_kernel).  Exact in exact arithmetic, for any centre tau0; each
// window takes the middle of its dates, where the polynomial's terms cancel
// least (the parts carry 48 bits each, so their rounding scales with the
// terms, not with the net curve).  The residual's response is ~1e-7 of the
// curve's stochastic part, so its FP32 rounding stays below 1e-14 of the
// curve.
//
// Windows.  The slots live in registers (kRespSlots of them).  A run with
// more dates is priced in launches over windows of dates [lo, hi], the latest
// window first: every launch evolves the parts and its window's slots from
// the first evolved step to date hi (the parts are cheap to repeat, the
// normals are counter-based), prices its dates, and passes to the next
// (earlier) window, per path, the sum of its cash flows and its part of the
// path's CVA contribution (carry [2][n_paths]); the earliest window (lo = 1)
// completes the path's CVA statistics.  Each window writes the EE partial
// sums and the exposure rows of its own dates.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>

#include "hjm_epilogue.cuh"
#include "hjm_eresp.h"
#include "hjm_resp.cuh"

namespace hjm {

// Groups of date slots that share one basic block with the step's normals
// and frame step (resp_groups_tail): two measured best (16.4 ms for the 10y
// headline against 17.3 ms with none, 16.4 with one, 16.5 with three; the
// reference table's cubic form 25.9 ms against 26.4 with one).
constexpr int kMergedGroups = 2;

namespace {

// Shared memory of one launch over window [lo, hi] (dates with a cash flow):
// cf_s [hi - lo + 3][kCta] (the epilogue's exposures alias it one row up),
// red_s, the parts' running sums z_s [NP][kCta], then the staged coefficient
// rows.
size_t eresp_smem(int lo, int hi, int np, int coef_floats4)
{
    return ((size_t)(hi - lo + 3) * kFp64Cta + 2 * (kFp64Cta / 32) + (size_t)np * kFp64Cta) * 8 +
           (size_t)coef_floats4 * 16;
}

// w = y_W + s n23 y_X in double-FP32 (the remainder's source W before step s
// of the block, NP = 4): the product's leading term exact by FMA, Knuth's
// two-sum for the addition, then renormalised.  The _rn intrinsics keep the
// compiler from fusing a product into a later addition, which would void the
// error-free transformations.
__device__ __forceinline__ void source_w(float sh, float sl, float xh, float xl, float wh, float wl, float& oh,
                                         float& ol)
{
    const float p = __fmul_rn(sh, xh);
    float e = fmaf(sh, xh, -p);
    e = fmaf(sh, xl, e);
    e = fmaf(sl, xh, e);
    const float s = __fadd_rn(wh, p);
    const float bp = __fsub_rn(s, wh);
    const float ap = __fsub_rn(s, bp);
    const float err = __fadd_rn(__fsub_rn(wh, ap), __fsub_rn(p, bp));
    const float l = __fadd_rn(wl, __fadd_rn(err, e));
    oh = __fadd_rn(s, l);
    ol = __fsub_rn(l, __fsub_rn(oh, s));
}

}  // namespace

// CTAs per SM of a kernel holding ns date slots: register-limited (24 slots
// in 168 registers, 16 or 20 in 128, 12 in 96, at 64 threads; 16 slots at 9
// CTAs per SM spill).
constexpr int eresp_min_ctas(int ns) { return ns >= 24 ? 6 : (ns >= 16 ? 8 : 10); }

// DEGS: the factors' polynomial degrees (degs_pack); NRES: the factors
// whose residual responses are in the table (0: none, one float4 per slot; 2:
// factors 2 and 3, two float4; 3: all three, three float4); SC: the frame's
// coefficient rows staged in shared memory; NS: date slots in registers (24,
// or 20, 16, 12 for windows with at most that many active slots: more CTAs
// per SM).  A date whose window slot is NS or beyond is never active (the
// host chose NS from the table's prefixes): its remainder is zero.
template <bool EXT, int DEGS, int NRES, bool SC, int NS = kRespSlots>
__global__ void __launch_bounds__(kFp64Cta, eresp_min_ctas(NS))
    path_kernel_fp64_eresp(const __grid_constant__ EulerRespParams E, const float4* __restrict__ resp,
                           const double* __restrict__ ext, double* __restrict__ partials,
                           double* __restrict__ estore, double* __restrict__ carry)
{
    constexpr int kCta = kFp64Cta;
    constexpr int NP = degs_parts(DEGS);
    constexpr int SR = frame_row(NP);
    constexpr int ENT = NRES == 3 ? 3 : (NRES == 2 ? 2 : 1);
    const PathParams<double>& P = E.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const int lo = E.win_lo, hi = E.win_hi;
    double* cf_s = reinterpret_cast<double*>(smem);
    double* red_s = cf_s + (size_t)(hi - lo + 3) * kCta;
    double* z_s = red_s + 2 * (kCta / 32);

    const int64_t cta_base = (int64_t)blockIdx.x * kCta;
    const int64_t lp = cta_base + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;

    // {remainder at tenor j, its running sum} as hi + lo pairs, slot hi - j
    float2 A[NS], Al[NS];
#pragma unroll
    for (int r = 0; r < NS; ++r) A[r] = Al[r] = make_float2(0.0f, 0.0f);
    float2 Y[NP], Yl[NP];  // the parts in the block's moving frame, {y_c, v_c} hi + lo
#pragma unroll
    for (int c = 0; c < NP; ++c) Y[c] = Yl[c] = make_float2(0.0f, 0.0f);
    const size_t rows = (size_t)B * P.stride;
    const int* nact = reinterpret_cast<const int*>(resp + rows * E.row * ENT);
    const float4* coef_g = resp + rows * E.row * ENT + (2 * rows + 5) / 4 + (size_t)E.frame_index * P.stride * SR;
    const float4* coef = coef_g;
    if constexpr (SC) {
        float4* c_s = reinterpret_cast<float4*>(z_s + NP * kCta);
        for (int i = tid; i < P.stride * SR; i += kCta) c_s[i] = coef_g[i];
        __syncthreads();
        coef = c_s;
    }
#pragma unroll
    for (int c = 0; c < NP; ++c) z_s[c * kCta + tid] = 0.0;

    const int roff = B - hi;                              // global slot of slot 0
    const int nslot0 = hi - (lo > 2 ? lo : 2) + 1;        // slots of this window's dates
    const int nslot = nslot0 < NS ? nslot0 : NS;          // those that can be active

    // price date i from its stochastic value xs and running sum zs
    auto price = [&](int i, double xs, double zs) {
        const double x = P.psamp[i] + xs;
        const double D = exp(-(P.psum[i] + zs) * P.dt);
        const double Lb = P.m * (exp(x * P.inv_m) - 1.0);
        cf_s[(size_t)(i - lo + 1) * kCta + tid] = D * (P.payA[i] * Lb - P.payB[i]);
    };

    // the normals of step n as hi + lo (lo = 0 for the generator's FP32 draws)
    auto draw = [&](int n, float (&h)[3], float (&l)[3]) {
        if constexpr (EXT) {
            double d0, d1, d2;
            draw_phi<double, true>(ext, gpath, active ? lp : 0, P.n_paths, n, P.rk0, P.rk1, d0, d1, d2);
            split_f64(d0, h[0], l[0]);
            split_f64(d1, h[1], l[1]);
            split_f64(d2, h[2], l[2]);
        } else {
            draw_phi<float, false>(ext, gpath, lp, P.n_paths, n, P.rk0, P.rk1, h[0], h[1], h[2]);
            l[0] = l[1] = l[2] = 0.0f;
        }
    };
    // Each step's normals are drawn one step ahead and, with the parts' frame
    // step that consumes the current ones, placed in the basic block of the
    // last groups of date slots (resp_groups_tail): the generator's and the
    // frame's dependent chains interleave with those groups'.  The step index
    // of the draw is clamped to the window's last evolved step (the draw after
    // it is discarded), which keeps external normals in bounds.
    const int n_last = hi * P.stride - 1;
    float ph[3], pl[3];
    if (hi > 1) draw(P.stride, ph, pl);

    if (lo == 1) price(1, 0.0, 0.0);  // the first block holds the curve at spot
    for (int b = 1; b < hi; ++b) {
        const float4* row = resp + ((size_t)b * P.stride * E.row + roff) * ENT;
        for (int s = 0; s < P.stride; ++s) {
            const int n = b * P.stride + s;
            int n_act = __ldg(nact + n) - roff;  // uniform: the row's active prefix in this window
            n_act = n_act < 0 ? 0 : (n_act > nslot ? nslot : n_act);
            // the prefix of the remainder's W terms (the residual's reaches further)
            int n_w = n_act;
            if constexpr (NRES > 0) {
                n_w = __ldg(nact + rows + 1 + n) - roff;
                n_w = n_w < 0 ? 0 : (n_w > nslot ? nslot : n_w);
            }
            const float4* rr = row + (size_t)s * E.row * ENT;
            // the remainder's source: W before this step's update
            float wh, wl;
            if constexpr (NP == 4) {
                const float4 sg = coef[(size_t)s * SR + 12];
                source_w(sg.x, sg.y, Y[3].x, Yl[3].x, Y[2].x, Yl[2].x, wh, wl);
            } else {
                wh = Y[2].x;
                wl = Yl[2].x;
            }
            const float2 wh2 = make_float2(wh, wh), wl2 = make_float2(wl, wl), nwh2 = make_float2(-wh, -wh);
            float nh[3], nl[3];
            resp_groups_tail<kMergedGroups>(n_act, [&](auto gc) {
                constexpr int G = decltype(gc)::value;
                if constexpr (4 * G < NS) {
                float4 k[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) k[u] = __ldg(rr + (4 * G + u) * ENT);
                if constexpr (NRES == 3) {
                    float4 r1[4], r2[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        r1[u] = __ldg(rr + (4 * G + u) * ENT + 1);
                        r2[u] = __ldg(rr + (4 * G + u) * ENT + 2);
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        float2& lo2 = Al[4 * G + u];
                        lo2 = __ffma2_rn(make_float2(r1[u].x, r1[u].y), make_float2(ph[0], ph[0]), lo2);
                        lo2 = __ffma2_rn(make_float2(r1[u].z, r1[u].w), make_float2(ph[1], ph[1]), lo2);
                        lo2 = __ffma2_rn(make_float2(r2[u].x, r2[u].y), make_float2(ph[2], ph[2]), lo2);
                    }
                } else if constexpr (NRES == 2) {
                    float4 r1[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) r1[u] = __ldg(rr + (4 * G + u) * ENT + 1);
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        float2& lo2 = Al[4 * G + u];
                        lo2 = __ffma2_rn(make_float2(r1[u].x, r1[u].y), make_float2(ph[1], ph[1]), lo2);
                        lo2 = __ffma2_rn(make_float2(r1[u].z, r1[u].w), make_float2(ph[2], ph[2]), lo2);
                    }
                }
                // (the merged groups, the latest dates, always: their W terms count)
                if (NRES == 0 || G < kMergedGroups || 4 * G < n_w) {
#pragma unroll
                    for (int u = 0; u < 4; ++u)
                        df_acc(A[4 * G + u], Al[4 * G + u], make_float2(k[u].x, k[u].y),
                               make_float2(k[u].z, k[u].w), wh2, wl2, nwh2);
                }
                }
            }, [&]() {
                draw(n < n_last ? n + 1 : n_last, nh, nl);
                // y += C(s) phi, v += G(s) phi for the (part, factor) terms of the degrees
                frame_step_n<DEGS, EXT, SC>(Y, Yl, coef + (size_t)s * SR, ph, pl);
            });
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                ph[k] = nh[k];
                pl[k] = nl[k];
            }
            // every fourth step, the active pairs renormalised (see renorm)
            if (E.renorm && (s & 3) == 3)
                resp_groups(n_act, [&](auto gc) {
                    constexpr int G = decltype(gc)::value;
                    if constexpr (4 * G < NS) {
#pragma unroll
                        for (int u = 0; u < 4; ++u) df_renorm(A[4 * G + u], Al[4 * G + u]);
                    }
                });
        }
        // the end of block b: the parts at date b + 1, priced when it is this window's
        double x[NP], Z[NP];
        frame_block_end_n<NP>(Y, Yl, E.frame, z_s + tid, kCta, x, Z);
        const int i = b + 1;
        if (i >= lo) {
            const double t = P.tau[i] - E.tau0;
            // (a slot beyond NS is never active: zero)
            float2 h = make_float2(0.0f, 0.0f), l = h;
            if (hi - i < NS) {
                h = select_reg<NS, float2>(A, hi - i);
                l = select_reg<NS, float2>(Al, hi - i);
            }
            double hc = widen_f32(h.x) + widen_f32(l.x);
            double hcs = widen_f32(h.y) + widen_f32(l.y);
            if (i == E.tenor_L) {  // (the basis-independent W = x[2] after the date's sampling step)
                hc = fma(E.wnew_L, x[2], hc);
                hcs = fma(E.wnew_L, x[2], hcs);
            }
            double px = x[NP - 1], pz = Z[NP - 1];
#pragma unroll
            for (int c = NP - 2; c >= 0; --c) {
                px = fma(t, px, x[c]);
                pz = fma(t, pz, Z[c]);
            }
            price(i, px + hc, pz + hcs);
        }
    }
    window_epilogue<kCta>(P, lo, hi, cf_s, red_s, partials, estore, carry, cta_base, lp, active);
}

// ---------------------------------------------------------------------------
// Tables
// ---------------------------------------------------------------------------
// Residual loadings r_k[t] of the table kernel, by value.
struct ResidLoadings {
    double r[kFactors][kMaxTenor];
};

// The responses of the remainder's source and of the residual loadings at the
// sampled tenors: entry (row b stride + s, slot r = B - j) holds, at lag
// l = (j - b) stride - 1 - s (the distance to date j's sampling step), the
// float4 {kappa G hi, kappa CG hi, kappa G lo, kappa CG lo} (each FP64 value
// split into the nearest float and the float nearest the rest) and, with the
// residual of all three factors (nres = 3), {R_j0, CR_j0, R_j1, CR_j1} and
// {R_j2, CR_j2, 0, 0} in FP32, or of factors 2 and 3 only (nres = 2, the
// first being an exact polynomial), {R_j1, CR_j1, R_j2, CR_j2}, for
// 1 <= b < j <= B.  Every lag of date j maps to one entry (q = j - b
// = l / stride + 1, s = q stride - 1 - l); the rest of the table stays zero.
// G and R by repeated upwind steps in FP64 (backward difference at the last
// tenor), one CTA per component (G, each residual factor), thread t holding
// tenor t.
__global__ void __launch_bounds__(kMaxTenor)
    eresp_table_kernel(int nt, double c, int stride, int B, int row, int nres, double kappa, ResidLoadings RL,
                       float4* __restrict__ resp)
{
    // CTA q: component 0 (kappa G, from e_L) or a residual factor's R_k (k = 0
    // with nres = 3; then 1 and 2), each with its running sum; the components
    // are independent, so they run on separate SMs (the recursion is FP64)
    const int k = nres == 3 ? (int)blockIdx.x - 1 : (int)blockIdx.x;  // residual factor of CTA q > 0
    __shared__ double v_s[kMaxTenor];
    const int t = threadIdx.x;
    const int L = nt - 1;
    const int M = (B - 1) * stride - 1;  // the longest lag read
    const int ent = nres == 3 ? 3 : (nres == 2 ? 2 : 1);
    double v = blockIdx.x == 0 ? ((t == L) ? 1.0 : 0.0) : (t < nt ? RL.r[k][t] : 0.0);
    double cum = 0.0;
    // the float2 of a residual factor: nres = 3: R_0 e[1].xy, R_1 e[1].zw,
    // R_2 e[2].xy; nres = 2: R_1 e[1].xy, R_2 e[1].zw
    const int f2 = nres == 3 ? k : k - 1;  // float2 index within the slot's entries after e[0]
    for (int m = 0; m <= M; ++m) {
        cum += v;
        if (t >= 2 && t <= B) {
            const int qd = m / stride + 1;
            const int b = t - qd;
            if (b >= 1) {
                float4* e = resp + (((size_t)b * stride + (size_t)(qd * stride - 1 - m)) * row + (B - t)) * ent;
                if (blockIdx.x == 0) {
                    const double g = kappa * v, cg = kappa * cum;
                    const float gh = __double2float_rn(g), cgh = __double2float_rn(cg);
                    e[0] = make_float4(gh, cgh, __double2float_rn(g - (double)gh), __double2float_rn(cg - (double)cgh));
                } else {
                    reinterpret_cast<float2*>(e + 1)[f2] = make_float2(__double2float_rn(v), __double2float_rn(cum));
                }
            }
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

// The remainder's responses under the predictor-corrector step (no residual:
// one float4 per slot, laid out as eresp_table_kernel's).  The two-stage
// step f' = A2 f + N (mu dt + xi) drives the remainder at L - 1 and L by W
// (the quadratic's boundary terms of A2 T^2 and N T^2): w0 W_old e_{L-1} +
// w1 W_old e_L + w2 W_new e_L with w0 = -c^2 dtau^2, w1 = wL - gL, w2 = gL
// (wL = -(2c + c^2) dtau^2, gL = -c dtau^2).  W_new of one step is W_old of
// the next, so the coefficient of the old W at lag l is H(l) = w0 G1(l) +
// w1 G2(l) + w2 G2(l + 1), with G1, G2 the responses of A2 to e_{L-1}, e_L
// (the three-point upwind stencil a0 = 1 - c + c^2/2, a1 = c - c^2,
// a2 = c^2/2, Euler rows at L - 1 and L), and its running sum likewise from
// the running sums of G1, G2.  FP64 recursion, thread t holding tenor t.
__global__ void __launch_bounds__(kMaxTenor)
    eresp_table_pc_kernel(int nt, double c, int stride, int B, int row, double w0, double w1, double w2,
                          float4* __restrict__ resp)
{
    __shared__ double v_s[kMaxTenor + 2], u_s[kMaxTenor + 2];
    const int t = threadIdx.x;
    const int L = nt - 1;
    const int M = (B - 1) * stride - 1;  // the longest lag read
    const double a0 = 1.0 - c + 0.5 * c * c, a1 = c - c * c, a2 = 0.5 * c * c;
    double g1 = (t == L - 1) ? 1.0 : 0.0, g2 = (t == L) ? 1.0 : 0.0;
    double cg1 = 0.0, cg2 = 0.0, hp = 0.0, chp = 0.0;  // H's first two terms at the previous lag
    for (int m = 0; m <= M + 1; ++m) {
        cg1 += g1;
        cg2 += g2;
        const int l = m - 1;  // the lag whose entry this iteration completes
        if (l >= 0 && t >= 2 && t <= B) {
            const int qd = l / stride + 1;
            const int b = t - qd;
            if (b >= 1) {
                const double g = hp + w2 * g2, cg = chp + w2 * cg2;
                const float gh = __double2float_rn(g), cgh = __double2float_rn(cg);
                resp[((size_t)b * stride + (size_t)(qd * stride - 1 - l)) * row + (B - t)] =
                    make_float4(gh, cgh, __double2float_rn(g - (double)gh), __double2float_rn(cg - (double)cgh));
            }
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

// Per row of the table (rows x row slots), two active prefixes in global
// slot numbering (slot r: date B - r): n_act[row], the slots up to the last
// one with any term that counts, and n_act[rows + 1 + row], up to the last
// one with a remainder term (kappa G, kappa CG) that counts.  A remainder
// term counts while it is at least 2^-53 |kappa| (for CG: 2^-53 |kappa|
// times the date's sampling step, the running sum's own unit): FP64's unit
// roundoff of the response G_L(0) = 1 of the last tenor to its own source.
// Away from the transport front the responses fall off faster than
// geometrically (binomial tails), so the terms one date drops sum to about
// ten times the threshold, ~1e-15 |kappa| max|W| (per running-sum unit): far
// under the slot's own double-FP32 rounding (2^-48 of the accumulator per
// addition), and 25% to 30% of the terms of a 10y or 12y run.  A residual
// term (R_jk, CR_jk) counts while it is at least 2^-60 of that component's
// largest magnitude anywhere in the table; the residual loadings reach every
// tenor, so its prefix covers nearly every date still to be sampled.  Zeros
// never count.  n_act[rows] = n_act[2 rows + 1] = 0 (read ahead).  One CTA.
__global__ void __launch_bounds__(1024)
    eresp_active_kernel(int rows, int row, int ent, int stride, int B, float kappa, const float4* __restrict__ resp,
                        int* __restrict__ n_act)
{
    __shared__ unsigned int mx[8];
    if (threadIdx.x < 8) mx[threadIdx.x] = 0u;
    __syncthreads();
    const int ncomp = ent == 3 ? 8 : (ent == 2 ? 6 : 2);
    auto comp = [&](size_t slot_base, int q) -> float {
        if (q < 2) {
            const float4 e = resp[slot_base];
            return q == 0 ? e.x : e.y;
        }
        const float4 e = resp[slot_base + (q < 6 ? 1 : 2)];
        switch (q) {
            case 2: return e.x;
            case 3: return e.y;
            case 4: return e.z;
            case 5: return e.w;
            case 6: return e.x;
            default: return e.y;
        }
    };
    const int64_t total = (int64_t)rows * row;
    if (ncomp > 2) {
        unsigned int m[6] = {0u, 0u, 0u, 0u, 0u, 0u};
        for (int64_t i = threadIdx.x; i < total; i += blockDim.x)
            for (int q = 2; q < ncomp; ++q)  // non-negative floats order as their bits
                m[q - 2] = max(m[q - 2], __float_as_uint(fabsf(comp((size_t)i * ent, q))));
        for (int q = 2; q < ncomp; ++q) atomicMax(&mx[q], m[q - 2]);
    }
    __syncthreads();
    const float tg = fabsf(kappa) * 0x1p-53f;
    for (int rw = threadIdx.x; rw <= rows; rw += blockDim.x) {
        int n = 0, ng = 0;
        if (rw < rows)
            for (int r = 0; r < row; ++r) {
                const float tcg = tg * (float)(max(B - r, 1) * stride);
                for (int q = 0; q < ncomp; ++q) {
                    const float a = fabsf(comp(((size_t)rw * row + r) * ent, q));
                    const float t = q == 0 ? tg : (q == 1 ? tcg : __uint_as_float(mx[q]) * 0x1p-60f);
                    if (a != 0.0f && a >= t) {
                        n = r + 1;
                        if (q < 2) ng = r + 1;
                    }
                }
            }
        n_act[rw] = n;
        n_act[rows + 1 + rw] = ng;
    }
}

// The moving-frame coefficients (hjm_resp.cuh): row s < stride, entry 3 c + k
// = {C hi, G hi, C lo, G lo} of C(s) = M^-(s+1) B and G(s) = Q(s) C(s), FP64
// split into the nearest float and the float nearest the rest; for NP = 4
// entry 12 = {sigma hi, sigma lo, 0, 0}, sigma = s n23 + sig0, the coefficient
// of y_X in the remainder's source before step s (W = y_W + s n23 y_X, plus
// the cubic's own share sig0 X).
struct FrameLoadings {
    PartsN n;
    double bm[4][kFactors];  // B[c][k]: loading of part c on factor k
    double sig0;
};

__global__ void eresp_coef_kernel(FrameLoadings f, int np, int stride, float4* __restrict__ coef)
{
    const int sr = frame_row(np);
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)stride * sr) return;
    const int64_t s = idx / sr;
    const int e = (int)(idx % sr);
    if (e == 12) {
        const double sg = fma((double)s, f.n.n23, f.sig0);
        const float h = __double2float_rn(sg);
        coef[idx] = make_float4(h, __double2float_rn(sg - (double)h), 0.0f, 0.0f);
        return;
    }
    const int c = e / 3, k = e % 3;
    if (c >= np) return;
    const double kk = (double)(s + 1), q = (double)s;
    // M^-k: c1 = -k, c2 = C(k+1, 2), c3 = -C(k+2, 3); Q(q): q I + C(q+1, 2) N + C(q+1, 3) N^2 + C(q+1, 4) N^3
    const PolyN minv(f.n, 1.0, -kk, 0.5 * kk * (kk + 1.0), -(kk + 2.0) * (kk + 1.0) * kk / 6.0);
    const PolyN Q(f.n, q, 0.5 * q * (q + 1.0), (q + 1.0) * q * (q - 1.0) / 6.0,
                  (q + 1.0) * q * (q - 1.0) * (q - 2.0) / 24.0);
    double b[4] = {0.0, 0.0, 0.0, 0.0}, C[4];
    for (int r = 0; r < np; ++r) b[r] = f.bm[r][k];
    for (int r = 0; r < 4; ++r) C[r] = minv.row(r, b);
    const double cv = C[c], gv = Q.row(c, C);
    const float ch = __double2float_rn(cv), gh = __double2float_rn(gv);
    coef[idx] = make_float4(ch, gh, __double2float_rn(cv - (double)ch), __double2float_rn(gv - (double)gh));
}

// ---------------------------------------------------------------------------
// Host
// ---------------------------------------------------------------------------
int eresp_row(int n_blocks) { return (n_blocks + 2 + 3) / 4 * 4; }

// The predictor-corrector's remainder source per unit W and step, w0 + w1 +
// w2 = -(2c + 2c^2) dtau^2 (the Euler step's kappa = -2 c dtau^2 to first order)
double eresp_kappa_pc(double c, double dtau) { return -(2.0 * c + 2.0 * c * c) * dtau * dtau; }

void eresp_make_frame(double dt, double dtau, int nt, const double (*svc)[3], const double* cubic,
                      const int* cubic_degs, double tau0, EulerRespFrame& fr, int& degs, bool pc)
{
    std::memset(&fr, 0, sizeof(fr));
    const double c = dt / dtau, sq = std::sqrt(dt);
    const double k1 = c * dtau, k2 = c * dtau * dtau;
    const double TL = dtau * (nt - 1);
    fr.tau0 = tau0;
    int dg[kFactors];
    if (cubic) {
        fr.np = 4;
        fr.n = PartsN{k1, k2, c * dtau * dtau * dtau, 2.0 * k1, 3.0 * k2, 3.0 * k1};
        fr.sig0 = 3.0 * (TL - tau0);
        // sum_e a_e (T - T_L)^e = sum_d a'_d (T - tau0)^d, a'_d = sum_{e>=d} C(e,d) a_e (tau0 - T_L)^(e-d)
        const double dl = tau0 - TL;
        for (int k = 0; k < kFactors; ++k) {
            const double* a = cubic + k * 4;
            const double sh[4] = {a[0] + dl * (a[1] + dl * (a[2] + dl * a[3])), a[1] + dl * (2.0 * a[2] + 3.0 * dl * a[3]),
                                  a[2] + 3.0 * dl * a[3], a[3]};
            for (int cc = 0; cc < 4; ++cc) fr.bm[cc][k] = sq * sh[cc];
            dg[k] = cubic_degs[k];
        }
    } else {
        fr.np = 3;
        fr.n = PartsN{k1, pc ? (c + c * c) * dtau * dtau : k2, 0.0, 2.0 * k1, 0.0, 0.0};
        fr.sig0 = 0.0;
        // sum_d s_d T^d = s'_0 + s'_1 t + s'_2 t^2 with t = T - tau0
        for (int k = 0; k < kFactors; ++k) {
            const double* a = svc[k];
            const double sh[3] = {a[0] + tau0 * (a[1] + tau0 * a[2]), a[1] + 2.0 * tau0 * a[2], a[2]};
            for (int cc = 0; cc < 3; ++cc) fr.bm[cc][k] = sh[cc];
            dg[k] = a[2] != 0.0 ? 2 : (a[1] != 0.0 ? 1 : 0);
        }
    }
    degs = degs_pack(dg[0], dg[1], dg[2]);
}

double eresp_window_centre(double dtau, int lo, int hi) { return 0.5 * dtau * (double)(lo + hi); }

int eresp_residual_factors(const double* resid, const double* vol, int nt)
{
    if (!resid) return 0;
    double r0 = 0.0, s0 = 0.0;
    for (int t = 0; t < nt; ++t) {
        r0 = std::max(r0, std::fabs(resid[t]));
        s0 = std::max(s0, std::fabs(vol[t]));
    }
    return r0 <= 0x1p-44 * s0 ? 2 : 3;
}

static int entries_per_slot(int nres) { return nres == 3 ? 3 : (nres == 2 ? 2 : 1); }

static size_t eresp_prefix_ints(int stride, int n_blocks) { return 2 * ((size_t)n_blocks * stride + 1); }

static size_t eresp_prefix_offset(int stride, int n_blocks, int nres)
{
    return (size_t)n_blocks * stride * eresp_row(n_blocks) * entries_per_slot(nres);
}

// (the kernel's coefficient rows start (2 rows + 5) / 4 float4 after the prefixes)
size_t eresp_table_elems(int stride, int n_blocks, int np, int nres, int n_frames)
{
    return eresp_prefix_offset(stride, n_blocks, nres) + (eresp_prefix_ints(stride, n_blocks) + 3) / 4 +
           (size_t)n_frames * stride * frame_row(np);
}

static cudaError_t launch_eresp_responses(int nt, double c, double dtau, int stride, int n_blocks, const double* resid,
                                   int nres, bool pc, float4* table, cudaStream_t s)
{
    if (nt < 3 || nt > kMaxTenor || n_blocks < 1 || n_blocks >= nt || stride < 1) return cudaErrorInvalidValue;
    const int row = eresp_row(n_blocks);
    if (!resid) nres = 0;
    const int ent = entries_per_slot(nres);
    const size_t rows = (size_t)n_blocks * stride;
    const size_t pre = eresp_prefix_offset(stride, n_blocks, nres);
    cudaError_t e = cudaMemsetAsync(table, 0, sizeof(float4) * (pre + (eresp_prefix_ints(stride, n_blocks) + 3) / 4), s);
    if (e != cudaSuccess) return e;
    ResidLoadings RL;
    std::memset(&RL, 0, sizeof(RL));
    if (resid)
        for (int k = 0; k < kFactors; ++k)
            for (int t = 0; t < nt; ++t) RL.r[k][t] = resid[k * nt + t];
    // kappa: the remainder's source per unit W and step, the scale of its
    // responses (the predictor-corrector's sources at L - 1 and L together)
    const double kappa = pc ? eresp_kappa_pc(c, dtau) : -2.0 * (c * dtau * dtau);
    if (pc) {
        if (nres != 0) return cudaErrorInvalidValue;
        const double d2 = dtau * dtau;
        eresp_table_pc_kernel<<<1, kMaxTenor, 0, s>>>(nt, c, stride, n_blocks, row, -c * c * d2, -(c + c * c) * d2,
                                                      -c * d2, table);
    } else {
        // one CTA for the remainder's responses, one per residual factor
        eresp_table_kernel<<<1 + nres, kMaxTenor, 0, s>>>(nt, c, stride, n_blocks, row, nres, kappa, RL, table);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    eresp_active_kernel<<<1, 1024, 0, s>>>((int)rows, row, ent, stride, n_blocks, (float)kappa, table,
                                            reinterpret_cast<int*>(table + pre));
    return cudaGetLastError();
}

static cudaError_t launch_eresp_frames(int stride, int n_blocks, int nres, const EulerRespFrame* frames, int n_frames,
                                float4* table, cudaStream_t s)
{
    if (n_frames < 1 || stride < 1) return cudaErrorInvalidValue;
    float4* coef = table + eresp_prefix_offset(stride, n_blocks, nres) + (eresp_prefix_ints(stride, n_blocks) + 3) / 4;
    const int64_t per_frame = (int64_t)stride * frame_row(frames[0].np);
    for (int w = 0; w < n_frames; ++w) {
        FrameLoadings f;
        std::memset(&f, 0, sizeof(f));
        f.n = frames[w].n;
        f.sig0 = frames[w].sig0;
        for (int cc = 0; cc < 4; ++cc)
            for (int k = 0; k < kFactors; ++k) f.bm[cc][k] = frames[w].bm[cc][k];
        eresp_coef_kernel<<<(unsigned)((per_frame + 127) / 128), 128, 0, s>>>(f, frames[0].np, stride,
                                                                               coef + w * per_frame);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_eresp_tables(int nt, double c, double dtau, int stride, int n_blocks, const EulerRespFrame* frames,
                                int n_frames, const double* resid, int nres, bool pc, float4* table, cudaStream_t s)
{
    if (!resid) nres = 0;
    const cudaError_t e = launch_eresp_responses(nt, c, dtau, stride, n_blocks, resid, nres, pc, table, s);
    if (e != cudaSuccess) return e;
    return launch_eresp_frames(stride, n_blocks, nres, frames, n_frames, table, s);
}

namespace {

template <bool EXT, int DEGS, int NRES>
cudaError_t launch_window(const EulerRespParams& E, int ns, const float4* table, const double* ext, double* partials,
                          double* estore, double* carry, cudaStream_t s)
{
    constexpr int NP = degs_parts(DEGS);
    const int sr = frame_row(NP);
    const bool sc = (size_t)E.P.stride * sr <= (size_t)kFrameSmemRows * kStateRow;
    const size_t smem = eresp_smem(E.win_lo, E.win_hi, NP, sc ? E.P.stride * sr : 0);
    auto k = sc ? path_kernel_fp64_eresp<EXT, DEGS, NRES, true> : path_kernel_fp64_eresp<EXT, DEGS, NRES, false>;
    // a window with at most 20, 16 or 12 dates that can be active, quadratic
    // factors, the generator's normals: fewer slots in fewer registers, more
    // CTAs per SM (the 10y headline: 12 slots, 10 CTAs, 12.9 ms against 13.6
    // with 20 slots at 8 CTAs; the cubic form with its residual spills at 128
    // registers and runs slower, 27.0 against 25.9 ms, and its residual keeps
    // every date still to be sampled active, so it keeps 24)
    // (with a residual table the windows hold 16 dates, eresp_window_dates: 16
    // slots in 126 registers, no spills, 8 CTAs per SM; the external-normals
    // variant spills there and keeps 24)
    if constexpr (!EXT && NRES > 0) {
        if (sc) k = path_kernel_fp64_eresp<EXT, DEGS, NRES, true, 16>;
    }
    if constexpr (!EXT && NRES == 0) {
        if (sc && ns <= 12)
            k = path_kernel_fp64_eresp<EXT, DEGS, NRES, true, 12>;
        else if (sc && ns <= 16)
            k = path_kernel_fp64_eresp<EXT, DEGS, NRES, true, 16>;
        else if (sc && ns <= 20)
            k = path_kernel_fp64_eresp<EXT, DEGS, NRES, true, 20>;
    }
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (E.P.n_paths + kFp64Cta - 1) / kFp64Cta;
    k<<<(unsigned)grid, kFp64Cta, smem, s>>>(E, table, ext, partials, estore, carry);
    return cudaGetLastError();
}

template <int DEGS, int NRES>
cudaError_t launch_window_ext(const EulerRespParams& E, int ns, const float4* table, const double* ext,
                              double* partials, double* estore, double* carry, cudaStream_t s)
{
    return ext ? launch_window<true, DEGS, NRES>(E, ns, table, ext, partials, estore, carry, s)
               : launch_window<false, DEGS, NRES>(E, ns, table, ext, partials, estore, carry, s);
}

}  // namespace

// The predictor-corrector's table (eresp_table_pc_kernel) restated in FP64
// on a unit grid (dtau = 1: every coefficient scales with dtau^2, as kappa).
static int eresp_first_active_date_pc(int nt, double c, int stride, int n_blocks)
{
    const int L = nt - 1, B = n_blocks;
    const double w0 = -c * c, w1 = -(c + c * c), w2 = -c, kap = std::fabs(eresp_kappa_pc(c, 1.0));
    const double a0 = 1.0 - c + 0.5 * c * c, a1 = c - c * c, a2 = 0.5 * c * c;
    double g1[kMaxTenor] = {}, g2[kMaxTenor] = {}, cg1[kMaxTenor] = {}, cg2[kMaxTenor] = {};
    double hp[kMaxTenor] = {}, chp[kMaxTenor] = {}, n1[kMaxTenor], n2[kMaxTenor];
    bool sig[kMaxTenor] = {};
    g1[L - 1] = 1.0;
    g2[L] = 1.0;
    const int M = (B - 1) * stride - 1;  // the longest lag in the table
    for (int m = 0; m <= M + 1; ++m) {
        for (int t = 0; t <= L; ++t) {
            cg1[t] += g1[t];
            cg2[t] += g2[t];
        }
        const int l = m - 1;
        // at half the device's thresholds (2^-53 |kappa|, times t stride for the running sum)
        if (l >= 0)
            for (int t = 2; t <= B; ++t)
                if (!sig[t] && l <= (t - 1) * stride - 1 &&
                    (std::fabs(hp[t] + w2 * g2[t]) >= 0x1p-54 * kap ||
                     std::fabs(chp[t] + w2 * cg2[t]) >= 0x1p-54 * kap * (double)t * stride))
                    sig[t] = true;
        for (int t = 0; t <= L; ++t) {
            hp[t] = w0 * g1[t] + w1 * g2[t];
            chp[t] = w0 * cg1[t] + w1 * cg2[t];
        }
        for (int t = 0; t < L - 1; ++t) {
            n1[t] = a0 * g1[t] + a1 * g1[t + 1] + a2 * g1[t + 2];
            n2[t] = a0 * g2[t] + a1 * g2[t + 1] + a2 * g2[t + 2];
        }
        n1[L - 1] = g1[L - 1] + c * (g1[L] - g1[L - 1]);
        n2[L - 1] = g2[L - 1] + c * (g2[L] - g2[L - 1]);
        n1[L] = g1[L] + c * (g1[L] - g1[L - 1]);
        n2[L] = g2[L] + c * (g2[L] - g2[L - 1]);
        for (int t = 0; t <= L; ++t) {
            g1[t] = n1[t];
            g2[t] = n2[t];
        }
    }
    for (int t = 2; t <= B; ++t)
        if (sig[t]) return t;
    return B + 1;
}

int eresp_first_active_date(int nt, double c, int stride, int n_blocks, int nres, bool pc)
{
    if (nres > 0) return 2;
    if (nt < 3 || nt > kMaxTenor || n_blocks < 2 || n_blocks >= nt || stride < 1) return 2;
    if (pc) return eresp_first_active_date_pc(nt, c, stride, n_blocks);
    const int L = nt - 1, B = n_blocks;
    double v[kMaxTenor] = {}, w[kMaxTenor], cum[kMaxTenor] = {};
    bool sig[kMaxTenor] = {};
    v[L] = 1.0;
    const int M = (B - 1) * stride - 1;  // the longest lag in the table
    for (int m = 0; m <= M; ++m) {
        for (int t = 0; t <= L; ++t) cum[t] += v[t];
        // date t's entries hold lags up to (t - 1) stride - 1; the device
        // counts kappa G >= 2^-53 |kappa|, kappa CG >= 2^-53 |kappa| t stride
        for (int t = 2; t <= B; ++t)
            if (!sig[t] && m <= (t - 1) * stride - 1 &&
                (std::fabs(v[t]) >= 0x1p-54 || std::fabs(cum[t]) >= 0x1p-54 * (double)t * stride))
                sig[t] = true;
        for (int t = 0; t < L; ++t) w[t] = v[t] + c * (v[t + 1] - v[t]);
        w[L] = v[L] + c * (v[L] - v[L - 1]);
        for (int t = 0; t <= L; ++t) v[t] = w[t];
    }
    for (int t = 2; t <= B; ++t)
        if (sig[t]) return t;
    return B + 1;
}

int eresp_windows(int n_blocks, int first_active, int* lo, int* hi, int* ns, int max_slots)
{
    const int f = std::max(first_active, 2);
    int n = 0, h = n_blocks;
    while (h >= 1) {
        // dates of a window [1, h] that can be active: f .. h
        int l = 1;
        if (h - f + 1 > max_slots) {
            l = h - max_slots + 1;
            if (l <= 2) l = 1;
        }
        const int act = std::max(h - std::max(l, f) + 1, 0);
        if (lo) lo[n] = l;
        if (hi) hi[n] = h;
        if (ns) ns[n] = act <= 12 ? 12 : (act <= 16 ? 16 : (act <= 20 ? 20 : kRespSlots));
        ++n;
        h = l - 1;
    }
    return n;
}

cudaError_t launch_path_fp64_eresp(const EulerRespParams& base, const EulerRespFrame* frames, int degs, int nres,
                                   const float4* table, int first_active, const double* ext, double* partials,
                                   double* estore, double* carry, cudaStream_t s, int* launches)
{
    int lo[kMaxTenor], hi[kMaxTenor], ns[kMaxTenor];
    const int nw = eresp_windows(base.P.n_blocks, first_active, lo, hi, ns, eresp_window_dates(nres));
    if (nw > 1 && !carry) return cudaErrorInvalidValue;
    if (launches) *launches = 0;
    for (int w = 0; w < nw; ++w) {
        EulerRespParams E = base;
        E.win_lo = lo[w];
        E.win_hi = hi[w];
        E.frame_index = w;
        E.n_frames = nw;
        E.tau0 = frames[w].tau0;
        cudaError_t e;
        if (nres == 2 && degs_of(degs, 0) == 0) {
            e = launch_window_ext<degs_pack(0, 3, 3), 2>(E, ns[w], table, ext, partials, estore, carry, s);
        } else if (nres > 0) {
            // (a residual table of factors 2 and 3 only is laid out as nres = 2)
            if (nres == 2) return cudaErrorInvalidValue;
            if (degs_of(degs, 0) == 0)
                e = launch_window_ext<degs_pack(0, 3, 3), 3>(E, ns[w], table, ext, partials, estore, carry, s);
            else
                e = launch_window_ext<degs_pack(3, 3, 3), 3>(E, ns[w], table, ext, partials, estore, carry, s);
        } else if (degs == degs_pack(0, 1, 2) || degs == degs_pack(0, 1, 1) || degs == degs_pack(0, 0, 2) ||
                   degs == degs_pack(0, 1, 0) || degs == degs_pack(0, 0, 1) || degs == degs_pack(0, 0, 0)) {
            e = launch_window_ext<degs_pack(0, 1, 2), 0>(E, ns[w], table, ext, partials, estore, carry, s);
        } else {
            e = launch_window_ext<degs_pack(2, 2, 2), 0>(E, ns[w], table, ext, partials, estore, carry, s);
        }
        if (e != cudaSuccess) return e;
        if (launches) ++*launches;
    }
    return cudaSuccess;
}

size_t eresp_max_smem(int n_blocks, int np, int stride, int first_active, int nres)
{
    int lo[kMaxTenor], hi[kMaxTenor];
    const int nw = eresp_windows(n_blocks, first_active, lo, hi, nullptr, eresp_window_dates(nres));
    const int sr = frame_row(np);
    const bool sc = (size_t)stride * sr <= (size_t)kFrameSmemRows * kStateRow;
    size_t m = 0;
    for (int w = 0; w < nw; ++w) m = std::max(m, eresp_smem(lo[w], hi[w], np, sc ? stride * sr : 0));
    return m;
}

}  // namespace hjm
