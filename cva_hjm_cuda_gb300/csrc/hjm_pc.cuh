// hjm_pc.cuh -- the predictor-corrector path state (hjm_pc.cu's valuation
// kernel and hjm_adjoint.cu's adjoint share it, so that the adjoint's forward
// pass repeats the valuation's arithmetic exactly).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "hjm_device.cuh"
#include "hjm_kernels.h"

namespace hjm {

constexpr int kPcCta = 64;

template <typename T>
__device__ __forceinline__ T exp_t(T x);
template <>
__device__ __forceinline__ double exp_t<double>(double x) { return exp(x); }
template <>
__device__ __forceinline__ float exp_t<float>(float x) { return expf(x); }
template <typename T>
__device__ __forceinline__ T expm1_t(T x);
template <>
__device__ __forceinline__ double expm1_t<double>(double x) { return exp(x) - 1.0; }
template <>
__device__ __forceinline__ float expm1_t<float>(float x) { return expm1f(x); }

// One path of the predictor-corrector scheme (the scheme and its growth
// scaling are described at the top of hjm_pc.cu): the growth-scaled stochastic
// curve v (POLY: its remainder) with its scale g, the polynomial parts, and the
// sums of a block for the discount recovery.  Shared memory columns of
// kPcCta threads: hs_s (NT rows) the curve at the block start, acc_s (B+1
// rows) the FP64 discount sums per tenor.
template <int NT, typename T, bool POLY>
struct PcPath {
    static constexpr int L = NT - 1;
    static constexpr int kGroup = 8;
    static constexpr int kGroups = (L - 1 + kGroup - 1) / kGroup;  // tenors 0 .. L-2
    T v[NT];
    T g, S, U, W;
    T F0, F1, F2, Tb;          // block sums of phi_k; anchor sum of v[L]
    T sS, sU, sW, XL1, XL;     // POLY: block sums of S, U, W and of the sources
    T ig;
    int live;                  // tenors <= live - 1 are never read again

    __device__ __forceinline__ void reset()
    {
#pragma unroll
        for (int t = 0; t < NT; ++t) v[t] = T(0);
        g = T(1);
        S = U = W = T(0);
    }
    __device__ __forceinline__ T poly_at(const PathParams<T>& P, T s_, T u_, T w_, int t) const
    {
        return POLY ? fma(P.tau[t], fma(P.tau[t], w_, u_), s_) : T(0);
    }
    // tenor i (runtime) of the stochastic curve
    __device__ __forceinline__ T value(const PathParams<T>& P, int i) const
    {
        return g * select_reg<NT, T>(v, i) + poly_at(P, S, U, W, i);
    }
    __device__ __forceinline__ void begin_block(const PathParams<T>& P, int b)
    {
        F0 = F1 = F2 = Tb = T(0);
        sS = sU = sW = XL1 = XL = T(0);
        ig = P.igblk[b];
        live = b + 1;
    }
    __device__ __forceinline__ void step(const PcParams<T>& Q, T phi0, T phi1, T phi2)
    {
        const PathParams<T>& P = Q.P;
        const T r1 = Q.r1, r2 = Q.r2;
        ig *= P.ip;
        const T p0 = phi0 * ig, p1 = phi1 * ig, p2 = phi2 * ig;
        auto noise = [&](int t) -> T { return fma(P.sv[2][t], p2, fma(P.sv[1][t], p1, P.sv[0][t] * p0)); };
        // the two Euler rows first (they read v[L-1], v[L]), then the
        // interior ascending in place (v[t+1], v[t+2] still old)
        const T eL = fma(T(2), v[L], -v[L - 1]);
        T vL1 = fma(r2, eL, fma(r1, v[L], v[L - 1]));
        T vL = fma(r2, fma(T(3), v[L], T(-2) * v[L - 1]), fma(r1, eL, v[L]));
        if constexpr (POLY) {
            // the remainder's sources (old W), then S, U, W (old values on the right)
            const T gam = fma(Q.aW[2], phi2, fma(Q.aW[1], phi1, Q.aW[0] * phi0));
            const T sL1 = Q.wL1 * W, sL = fma(Q.gL, gam, Q.wL * W);
            vL1 = fma(sL1, ig, vL1);
            vL = fma(sL, ig, vL);
            XL1 += sL1;
            XL += sL;
            T Sn = fma(Q.aS[0], phi0, fma(Q.k2p, W, fma(Q.k1, U, S)));
            Sn = fma(Q.aS[2], phi2, fma(Q.aS[1], phi1, Sn));
            const T Un = fma(Q.aU[2], phi2, fma(Q.aU[1], phi1, fma(Q.aU[0], phi0, fma(Q.k1x2, W, U))));
            S = Sn;
            U = Un;
            W += gam;
            sS += S;
            sU += U;
            sW += W;
        } else {
            vL1 += noise(L - 1);
            vL += noise(L);
            F0 += phi0;
            F1 += phi1;
            F2 += phi2;
        }
#pragma unroll
        for (int gi = 0; gi < kGroups; ++gi) {
            if (kGroup * gi + kGroup > live) {
#pragma unroll
                for (int j = 0; j < kGroup; ++j) {
                    const int t = kGroup * gi + j;
                    if (t <= L - 2) {
                        T x = v[t];
                        if constexpr (!POLY) {
                            x = fma(P.sv[0][t], p0, x);
                            x = fma(P.sv[1][t], p1, x);
                            x = fma(P.sv[2][t], p2, x);
                        }
                        x = fma(r1, v[t + 1], x);
                        v[t] = fma(r2, v[t + 2], x);
                    }
                }
            }
        }
        v[L - 1] = vL1;
        v[L] = vL;
        Tb = fma(P.ip, Tb, v[L]);
    }
    // end of block b: the scale at the block end, the block sums of tenors
    // b+1 .. B folded into acc_s (downward from the anchor H[L] = g Tb), and
    // the block-end curve into hs_s (the next block's start)
    __device__ __forceinline__ void end_block(const PcParams<T>& Q, int b, int B, T* hs_s, double* acc_s, int tid)
    {
        const PathParams<T>& P = Q.P;
        g = P.gblk[b + 1];  // base^-(b stride)
        auto X = [&](int t) -> T {
            if constexpr (POLY) return t == L - 1 ? XL1 : (t == L ? XL : T(0));
            return fma(P.sv[2][t], F2, fma(P.sv[1][t], F1, P.sv[0][t] * F0));
        };
        const T dL = fma(g, v[L], -hs_s[L * kPcCta + tid]);
        const T dL1 = fma(g, v[L - 1], -hs_s[(L - 1) * kPcCta + tid]);
        const T HL = g * Tb;
        const T HL1 = fma(X(L - 1) - fma(Q.ce, dL - dL1, dL1), Q.inv_ce, HL);
        if (L <= B) acc_s[L * kPcCta + tid] += as_f64(HL + poly_at(P, sS, sU, sW, L));
        if (L - 1 <= B && L - 1 > b) acc_s[(L - 1) * kPcCta + tid] += as_f64(HL1 + poly_at(P, sS, sU, sW, L - 1));
        T H1 = HL1, H2 = HL, d1 = dL1, d2 = dL;
#pragma unroll
        for (int t = L - 2; t >= 1; --t) {
            if (t <= b) break;
            const T d = fma(g, v[t], -hs_s[t * kPcCta + tid]);
            const T a2d = fma(Q.a2e, d2, fma(Q.a1e, d1, Q.a0e * d));
            const T Ht = (X(t) - a2d + fma(Q.a1e, H1, Q.a2e * H2)) * Q.inv_1ma0;
            if (t <= B) acc_s[t * kPcCta + tid] += as_f64(Ht + poly_at(P, sS, sU, sW, t));
            H2 = H1;
            H1 = Ht;
            d2 = d1;
            d1 = d;
        }
#pragma unroll
        for (int t = 0; t < NT; ++t) hs_s[t * kPcCta + tid] = g * v[t];
    }
};

}  // namespace hjm
