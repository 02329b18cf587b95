// hjm_pairs.cuh -- packed FP32x2 helpers shared by the mixed-precision path
// kernel and the adjoint kernel.
//
// The curve of one path is held as H = ceil(NT/2) float2 pairs, pair p =
// {h[p], h[p+H]}; both upwind neighbours (h[t+1] in the Euler step, g[t-1] in
// its adjoint) of nearly every tenor lie in the same component of the next or
// previous pair, so one packed FMA (__ffma2_rn) serves two tenors.
#pragma once

#include <cuda_runtime.h>

#include "hjm_device.cuh"
#include "hjm_kernels.h"

namespace hjm {

template <int NT>
struct PairGrid {
    static constexpr int H = (NT + 1) / 2;  // pairs
    static constexpr int L = NT - 1;        // last tenor
};

// One growth-scaled Euler step of the packed curve v (table volatility): with
// the normals already scaled by (1 + rr)^(n'+1) (p0..p2),
//   v'[t] = v[t] + sum_k sv[k][t] p_k + rr v[t+1],        t < L,
//   v'[L] = v[L] + sum_k sv[k][L] p_k + rr (2 v[L] - v[L-1]),
// four packed FMAs per pair of tenors.  The seam pair (p = H-1, whose .x
// neighbour is pair 0's .y), the pair holding the last tenor and the padding
// tenor of an odd grid take scalar fix-ups.
template <int NT>
__device__ __forceinline__ void euler_step_pairs(float2 (&h)[PairGrid<NT>::H], const MixedParams& M, float p0,
                                                 float p1, float p2)
{
    constexpr int H = PairGrid<NT>::H, L = PairGrid<NT>::L;
    const float2 f0 = make_float2(p0, p0), f1 = make_float2(p1, p1), f2 = make_float2(p2, p2);
    const float rr = M.P.rr;
    float2 hn[H];
#pragma unroll
    for (int p = 0; p < H; ++p) {
        const int q = H + p;  // tenor held in .y
        if (p + 1 < H && q < L) {
            float2 x = __ffma2_rn(M.svp[0][p], f0, h[p]);
            x = __ffma2_rn(M.svp[1][p], f1, x);
            x = __ffma2_rn(M.svp[2][p], f2, x);
            hn[p] = __ffma2_rn(M.rp, h[p + 1], x);
        } else {
            float x = fmaf(M.svp[2][p].x, p2, fmaf(M.svp[1][p].x, p1, fmaf(M.svp[0][p].x, p0, h[p].x)));
            hn[p].x = fmaf(rr, (p + 1 < H) ? h[p + 1].x : h[0].y, x);
            if (q < L) {
                x = fmaf(M.svp[2][p].y, p2, fmaf(M.svp[1][p].y, p1, fmaf(M.svp[0][p].y, p0, h[p].y)));
                hn[p].y = fmaf(rr, h[p + 1].y, x);
            } else if (q == L) {
                x = fmaf(M.svp[2][p].y, p2, fmaf(M.svp[1][p].y, p1, fmaf(M.svp[0][p].y, p0, h[p].y)));
                hn[p].y = fmaf(rr, fmaf(2.0f, h[p].y, -h[p - 1].y), x);
            } else {
                hn[p].y = 0.0f;  // padding tenor of an odd grid: stays zero
            }
        }
    }
#pragma unroll
    for (int p = 0; p < H; ++p) h[p] = hn[p];
}

template <int NT>
__device__ __forceinline__ float select_pair(const float2 (&h)[PairGrid<NT>::H], int i)
{
    constexpr int H = PairGrid<NT>::H;
    float r = 0.0f;
#pragma unroll
    for (int p = 0; p < H; ++p) {
        r = (p == i) ? h[p].x : r;
        r = (p + H == i) ? h[p].y : r;
    }
    return r;
}

// Tenor t (compile-time after unrolling) of a packed curve.
template <int NT>
__device__ __forceinline__ float pair_tenor(const float2 (&h)[PairGrid<NT>::H], int t)
{
    constexpr int H = PairGrid<NT>::H;
    return t < H ? h[t].x : h[t - H].y;
}

// Block-sum recovery in FP32, upwards from the anchor tenor 1.  Over a run of
// Euler steps, with Phi_k the sums of the normals, H1 the sum of h[1] and
// d = h_now - h_start (h_now = gs * v, h_start in hs_s, thread column tid,
// stride cta),
//     H[t+1] = H[t] + ((A d)[t] - sum_k sv[k][t] Phi_k) / c,   t = 1 .. tmax-1,
// and fold(t, H[t]) is called for t = 2 .. tmax (tmax <= NT-1).
template <int NT, typename Fold>
__device__ __forceinline__ void recover_sums_up(const float2 (&h)[PairGrid<NT>::H], const float* hs_s, int tid,
                                                int cta, const PathParams<float>& P, float gs, float F0, float F1,
                                                float F2, float H1, int tmax, Fold fold)
{
    const float c = P.c, inv_c = (float)P.inv_c;
    float Hn = H1;
    float d = fmaf(gs, pair_tenor<NT>(h, 1), -hs_s[1 * cta + tid]);
#pragma unroll
    for (int t = 1; t < NT - 1; ++t) {
        if (t >= tmax) break;
        const float dn = fmaf(gs, pair_tenor<NT>(h, t + 1), -hs_s[(t + 1) * cta + tid]);
        const float xi = fmaf(P.sv[2][t], F2, fmaf(P.sv[1][t], F1, P.sv[0][t] * F0));
        const float ad = fmaf(c, dn - d, d);
        Hn = fmaf(ad - xi, inv_c, Hn);
        fold(t + 1, Hn);
        d = dn;
    }
}

// The growth-scaled convection of the packed curve (polynomial volatility:
// the noise lives in the scalar parts S, U, W), with the last-tenor source
// src already scaled by (1 + rr)^(n'+1): one packed FMA per pair of tenors.
template <int NT>
__device__ __forceinline__ void convect_pairs(float2 (&h)[PairGrid<NT>::H], const MixedParams& M, float src)
{
    constexpr int H = PairGrid<NT>::H, L = PairGrid<NT>::L;
    const float rr = M.P.rr;
    float2 hn[H];
#pragma unroll
    for (int p = 0; p < H; ++p) {
        const int q = H + p;
        if (p + 1 < H && q < L) {
            hn[p] = __ffma2_rn(M.rp, h[p + 1], h[p]);
        } else {
            hn[p].x = fmaf(rr, (p + 1 < H) ? h[p + 1].x : h[0].y, h[p].x);
            if (q < L)
                hn[p].y = fmaf(rr, h[p + 1].y, h[p].y);
            else if (q == L)
                hn[p].y = fmaf(rr, fmaf(2.0f, h[p].y, -h[p - 1].y), h[p].y) + src;
            else
                hn[p].y = 0.0f;
        }
    }
#pragma unroll
    for (int p = 0; p < H; ++p) h[p] = hn[p];
}

// One path's stochastic curve in mixed precision.  Table volatility: the packed
// curve h itself.  Polynomial volatility (POLY, degree <= 2): h = S 1 + U T +
// W T^2 + hc, with the packed hc only convected (see the FP64 kernel for the
// algebra: A 1 = 1, A T = T + c dtau 1, A T^2 = T^2 + 2 c dtau T + c dtau^2 1
// - 2 c dtau^2 e_L).  CUB (a table that is a cubic up to a residual below
// FP32's resolution of it, such as the reference driver's own PCA table): a
// fourth part X of T^3, with T the tenor minus the basis centre (P.tau holds
// it), A T^3 = T^3 + 3 c dtau T^2 + 3 c dtau^2 T + c dtau^3 1 in the interior,
// and the remainder's source at the last tenor -2 c dtau^2 (W + 3 T_L X).
template <int NT, bool POLY, bool CUB = false>
struct MixedPath {
    static_assert(!CUB || POLY, "the cubic part extends the polynomial form");
    static constexpr int H = PairGrid<NT>::H;
    float2 h[H];  // v = h / g (POLY: the convected remainder hc, scaled alike)
    float S, U, W, X;
    float g;      // (1 + rr)^-n', n' = steps evolved so far
    float ig;     // (1 + rr)^n' (POLY: times -2 c dtau^2, the source per unit W)

    __device__ __forceinline__ void reset()
    {
#pragma unroll
        for (int p = 0; p < H; ++p) h[p] = make_float2(0.f, 0.f);
        S = U = W = X = 0.f;
        g = ig = 1.f;
    }
    // the scales at the start of block b, from the table (no drift across blocks)
    __device__ __forceinline__ void begin_block(const PathParams<float>& P, int b)
    {
        g = P.gblk[b];
        ig = POLY ? P.m2k2 * P.igblk[b] : P.igblk[b];
    }
    __device__ __forceinline__ void step(const MixedParams& M, float phi0, float phi1, float phi2)
    {
        ig *= M.P.ip;
        if constexpr (POLY) {
            convect_pairs<NT>(h, M, ig * (CUB ? fmaf(M.src3f, X, W) : W));
            // the noise projection folded into the updates (old U, W, X on the right)
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
            }
            S = Sn;
            U = Un;
            W = Wn;
        } else {
            euler_step_pairs<NT>(h, M, phi0 * ig, phi1 * ig, phi2 * ig);
        }
        g *= M.P.qm;
    }
    // the polynomial part at basis coordinate t
    __device__ __forceinline__ float poly(float t) const
    {
        return CUB ? fmaf(t, fmaf(t, fmaf(t, X, W), U), S) : fmaf(t, fmaf(t, W, U), S);
    }
    // tenor i (runtime) of the stochastic curve
    __device__ __forceinline__ float value(const PathParams<float>& P, int i) const
    {
        float v = g * select_pair<NT>(h, i);
        if (POLY) v += poly(P.tau[i]);
        return v;
    }
    // tenor t (compile-time after unrolling) of the stochastic curve without
    // the polynomial part
    __device__ __forceinline__ float rem(int t) const { return g * pair_tenor<NT>(h, t); }
};

// Running sums over a block (or a partial block) of steps for the recovery.
struct BlockSums {
    float F0, F1, F2, H1, sS, sU, sW, sX;
    __device__ __forceinline__ void reset() { F0 = F1 = F2 = H1 = sS = sU = sW = sX = 0.f; }
    template <int NT, bool POLY, bool CUB>
    __device__ __forceinline__ void add(const MixedPath<NT, POLY, CUB>& x, float phi0, float phi1, float phi2)
    {
        if constexpr (POLY) {
            sS += x.S;
            sU += x.U;
            sW += x.W;
            if constexpr (CUB) sX += x.X;
        } else {
            F0 += phi0;
            F1 += phi1;
            F2 += phi2;
        }
        H1 = fmaf(x.g, x.h[1].x, H1);
    }
    // the block sums of the polynomial part at basis coordinate t
    template <bool CUB>
    __device__ __forceinline__ float poly(float t) const
    {
        return CUB ? fmaf(t, fmaf(t, fmaf(t, sX, sW), sU), sS) : fmaf(t, fmaf(t, sW, sU), sS);
    }
};

// Block sums of tenors 2 .. tmax of the stochastic curve over the steps the
// sums cover (upward recovery from tenor 1 plus, POLY, the scalar parts);
// fold(t, sum) is called for t = 2 .. tmax.
template <int NT, bool POLY, bool CUB, typename Fold>
__device__ __forceinline__ void block_sums_up(const MixedPath<NT, POLY, CUB>& x, const float* hs_s, int tid, int cta,
                                              const PathParams<float>& P, const BlockSums& bs, int tmax, Fold fold)
{
    if constexpr (POLY) {
        recover_sums_up<NT>(x.h, hs_s, tid, cta, P, x.g, 0.f, 0.f, 0.f, bs.H1, tmax, [&](int t, float Ht) {
            fold(t, Ht + bs.poly<CUB>(P.tau[t]));
        });
    } else {
        recover_sums_up<NT>(x.h, hs_s, tid, cta, P, x.g, bs.F0, bs.F1, bs.F2, bs.H1, tmax, fold);
    }
}

// One growth-scaled reverse step on the packed adjoint state.  The adjoint
// obeys g <- A^T (g + inj) with A^T, per tenor (L the last tenor):
//   t = 0:          (1 - c) g[0]
//   1 <= t <= L-2:  (1 - c) g[t] + c g[t-1]
//   t = L-1:        (1 - c) g[t] + c (g[t-1] - g[L])
//   t = L:          (1 + c) g[L] + c g[L-1].
// Holding gs = g (1 + rr)^k after k steps of a block (rr = c / (1 - c), the
// forward's constant), the step is gs <- Ahat (gs + sig inj) with sig =
// (1 + rr)^k and Ahat = A^T / (1 - c):
//   G[t] + rr G[t-1],  G[L-1] + rr (G[L-2] - G[L]),  G[L] + rr (2 G[L] + G[L-1]),
// one packed FMA for the seeds and one for the step per pair of tenors.
template <int NT>
__device__ __forceinline__ void adjoint_step_pairs(float2 (&g)[PairGrid<NT>::H], const float2 (&inj)[PairGrid<NT>::H],
                                                   float sig, float rr, float& G_last)
{
    constexpr int H = PairGrid<NT>::H, L = PairGrid<NT>::L;
    const float2 ss = make_float2(sig, sig), rp = make_float2(rr, rr);
    // streamed in ascending pairs with the previous pair's G in registers; the
    // two values needed ahead of their pair (tenor H-1 for the seam, tenor L
    // for row L-1) are formed first
    const float G_seam = fmaf(inj[H - 1].x, sig, g[H - 1].x);
    G_last = fmaf(inj[L - H].y, sig, g[L - H].y);
    float2 Gprev = make_float2(0.f, 0.f);
#pragma unroll
    for (int p = 0; p < H; ++p) {
        const int q = H + p;
        const float2 Gp = __ffma2_rn(inj[p], ss, g[p]);
        if (p >= 1 && q < L - 1) {
            g[p] = __ffma2_rn(rp, Gprev, Gp);
        } else {
            g[p].x = (p == 0) ? Gp.x : fmaf(rr, Gprev.x, Gp.x);
            const float gprev = (p == 0) ? G_seam : Gprev.y;  // tenor q-1
            if (q < L - 1)
                g[p].y = fmaf(rr, gprev, Gp.y);
            else if (q == L - 1)
                g[p].y = fmaf(rr, gprev - G_last, Gp.y);
            else if (q == L)
                g[p].y = fmaf(rr, fmaf(2.0f, Gp.y, gprev), Gp.y);
            else
                g[p].y = 0.0f;  // padding tenor
        }
        Gprev = Gp;
    }
}

}  // namespace hjm
