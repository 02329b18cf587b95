// hjm_resp.cuh -- device helpers of the FP64 response forms.
//
// The date-slot dispatch (groups of four slots, Duff's device), the
// double-FP32 helpers and the polynomial parts' moving frame shared by the
// Euler and predictor-corrector response form (path_kernel_fp64_eresp in
// hjm_eresp.cu), and the slot constants of the volatility-table response form
// (path_kernel_fp64_vresp in hjm_forward.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <type_traits>

#include "hjm_kernels.h"

namespace hjm {

// Response form.  The remainder hc of the polynomial decomposition starts at
// zero, is driven only at the last tenor (Euler: by kappa W_{n-1} at step n,
// kappa = -2 c dtau^2, W before the step's update; the predictor-corrector
// step drives it at L - 1 and L by W before and after the step) and is
// otherwise convected by the scheme's A.  So after step K its value at tenor
// j and its running sum are fixed linear functionals of the W history,
//     hc_K[j]               = sum_{n<=K} H_j(K - n)  W_{n-1},
//     sum_{K'<=K} hc_K'[j]  = sum_{n<=K} CH_j(K - n) W_{n-1},
// (Euler: H_j(m) = kappa (A^m e_L)[j]), exact in exact arithmetic.  The
// pricing reads hc only at tenor j at date j's sampling step K_j = j stride
// - 1 (its value and, for the discount, its running sum), so the kernel keeps
// those two numbers per date still to be sampled and adds one term to each
// per step, in place of the convection of every live tenor and the block-end
// discount recovery.  H_j(m) vanishes while the lag m is too short for the
// transport from the last tenor to reach tenor j (one tenor per step under
// Euler, two under the predictor-corrector's stencil).
//
// Both sums are carried in double-FP32 arithmetic on the FP32 pipe (76 times
// the FP64 pipe's rate on GB300): the table holds each coefficient as a pair
// of floats hi + lo (48 significant bits), W is the parts' own double-FP32
// accumulator, the product's leading term is made exact by an FMA and the
// accumulation by Knuth's two-sum (df_acc), packed {value, running sum} in
// FP32x2 instructions.  The relative error of a date's sum stays below ~1e-12
// of its magnitude (checked against FP64 sums of the same terms), and the
// remainder at a sampled tenor is a small part of the curve (the far tail of
// the transport from the last tenor), so its rounding stays within an ulp of
// the FP64 curve.
//
// The accumulators of date j sit in slot r = B - j (of the window).  At step
// s of block b the dates with a term that counts form a prefix of the slots,
// n_act of them, which the kernels read per row from the table (its active
// prefix, eresp_active_kernel).  A switch on the number of groups of four
// slots covering it enters a fall-through chain of groups (Duff's device):
// the skipped groups issue nothing (a predicated loop would issue them all),
// and the four terms of a group form one basic block, their loads in flight
// together and their FP32 chains interleaved.  The table is zero outside the
// live nonzero entries, so the slots a group adds beyond n_act add exact
// zeros (dead or not yet reached dates).
constexpr int kRespDates = 24;   // dates a response-form window holds (one launch of hjm_run_static)
constexpr int kRespSlots = 24;   // accumulator slots, a multiple of the group of 4 (slot 23 stays zero)
constexpr int kRespRow = 24;     // response-table row: one float4 per slot

// A double as hi + lo + O(2^-47 |d|), hi and lo FP32, with integer
// operations only (conversion and arithmetic instructions on doubles issue on
// the FP64 pipe): hi is d with its significand truncated to 24 bits, lo the
// remaining 29 bits, converted (rounded to 24 bits) and scaled by 2^(E - 52).
// |d| below 2^-126 gives zeros, lo below the FP32 normal range is dropped
// (|d| < 2^-74: then hi alone, within 2^-23), |d| above 2^128 saturates.
__device__ __forceinline__ void split_f64(double d, float& hi, float& lo)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    const uint32_t top = (uint32_t)(u >> 32);
    const uint32_t sign = top & 0x80000000u;
    const int e = (int)((top >> 20) & 0x7ffu);  // biased FP64 exponent
    const int eh = e - 1023 + 127;               // biased FP32 exponent of hi
    if (eh <= 0) {
        hi = lo = __uint_as_float(sign);
        return;
    }
    if (eh > 254) {
        hi = __uint_as_float(sign | 0x7f7fffffu);
        lo = __uint_as_float(sign);
        return;
    }
    hi = __uint_as_float(sign | ((uint32_t)eh << 23) | ((uint32_t)(u >> 29) & 0x7fffffu));
    const uint32_t r = (uint32_t)u & 0x1fffffffu;  // the truncated bits, in units of 2^(E - 52)
    const float scale = (eh > 52) ? __uint_as_float((uint32_t)(eh - 52) << 23) : 0.0f;
    lo = __uint_as_float(sign | __float_as_uint((float)r * scale));
}

// -v in both lanes (folded into the consumer's operand)
__device__ __forceinline__ float2 neg2(float2 v) { return make_float2(-v.x, -v.y); }

// (A, Al) += (kh + kl) (wh + wl) in double-FP32, both lanes: the product's
// leading term exact by FMA, the cross terms in FP32, kl wl (2^-48) dropped;
// Knuth's two-sum keeps A + Al exact up to the FP32 rounding of Al.  nwh =
// -wh (formed once per step by the caller): the product is taken negated,
// pn = -fl(kh wh), so that the exact error kh wh - fl(kh wh) is one FMA with
// pn as the addend and no instruction negates a product; every rounding is
// that of the plain formulation (negation is exact).
__device__ __forceinline__ void df_acc(float2& A, float2& Al, float2 kh, float2 kl, float2 wh, float2 wl, float2 nwh)
{
    const float2 pn = __fmul2_rn(kh, nwh);
    float2 e = __ffma2_rn(kh, wh, pn);
    e = __ffma2_rn(kh, wl, e);
    e = __ffma2_rn(kl, wh, e);
    const float2 sum = __fadd2_rn(A, neg2(pn));   // A + p
    const float2 bp = __fadd2_rn(sum, neg2(A));   // sum - A
    const float2 ap = __fadd2_rn(sum, neg2(bp));  // sum - bp
    // (A - ap) + (p - bp), with p - bp = -(pn + bp)
    const float2 err = __fadd2_rn(__fadd2_rn(A, neg2(ap)), neg2(__fadd2_rn(pn, bp)));
    Al = __fadd2_rn(Al, __fadd2_rn(err, e));
    A = sum;
}

// (A, Al) += (kh + kl) w for w exact in FP32 (a normal draw), nw = -w:
// df_acc without the w_lo term.
__device__ __forceinline__ void df_acc_w(float2& A, float2& Al, float2 kh, float2 kl, float2 w, float2 nw)
{
    const float2 pn = __fmul2_rn(kh, nw);
    float2 e = __ffma2_rn(kh, w, pn);
    e = __ffma2_rn(kl, w, e);
    const float2 sum = __fadd2_rn(A, neg2(pn));
    const float2 bp = __fadd2_rn(sum, neg2(A));
    const float2 ap = __fadd2_rn(sum, neg2(bp));
    const float2 err = __fadd2_rn(__fadd2_rn(A, neg2(ap)), neg2(__fadd2_rn(pn, bp)));
    Al = __fadd2_rn(Al, __fadd2_rn(err, e));
    A = sum;
}

// (A, Al) renormalised: A = fl(A + Al) and Al the rest (Dekker's fast
// two-sum, exact when |A| >= |Al| or A = 0, which the accumulators keep: Al
// only gathers rounding errors of A).  Done after every step's terms, it
// keeps |Al| <= ulp(A) / 2, so that the FP32 rounding of the low parts stays
// at 2^-48 of A per addition instead of growing with the number of terms.
__device__ __forceinline__ void df_renorm(float2& A, float2& Al)
{
    const float2 sum = __fadd2_rn(A, Al);
    Al = __fadd2_rn(Al, neg2(__fadd2_rn(sum, neg2(A))));  // Al - (sum - A)
    A = sum;
}

// Polynomial parts in a moving frame (the FP64 response forms of both
// schemes).  A step maps the parts x = (S, U, W) of h's quadratic to
// M x + B phi with M = I + N, N = [[0, n01, n02], [0, 0, n12], [0, 0, 0]] (the
// scheme's difference operator on a quadratic, which it takes exactly:
// Euler n01 = c dtau, n02 = c dtau^2, n12 = 2 c dtau; predictor-corrector
// n01 = c dtau, n02 = (c + c^2) dtau^2, n12 = 2 c dtau) and B[c][k] the
// loading of part c on factor k.  M is unipotent (N^3 = 0), so within a
// block, anchored at its first step (y_0 = x at the block's start), y_s =
// M^-s x moves by the noise alone,
//     y_{s+1} = y_s + C(s) phi_s,                  C(s) = M^-(s+1) B,
// and at the block's end (s = a = stride)
//     x_end = M^a y_a,
//     sum_{s'=1..a} x_s' = Q(a) y_a - v,            v = sum_s G(s) phi_s,
// with Q(a) = sum_{e=1..a} M^e, G(s) = Q(s) C(s), and (N^2 has the one entry
// n01 n12 at (S, W))
//     M^a   = I + a N + a(a-1)/2 N^2,
//     M^-k  = I - k N + k(k+1)/2 N^2,
//     Q(a)  = a I + a(a+1)/2 N + (a+1)a(a-1)/6 N^2.
// Per step the kernels add C(s) phi to y and G(s) phi to v (6 terms for
// factors of degree <= k, 9 in general), packed {y, v} per part in
// double-FP32 on the FP32 pipe, and renormalise the pairs (df_renorm); at
// each block's end (a sampling date) they widen them, form x_end, add the
// block's sum to the running sums Z in FP64, and re-anchor y on x_end
// (rounded to FP32 pairs) with v = 0.  The coefficients
// are the same in every block: row s (< stride) of the coefficient table
// holds kStateRow float4 {C hi, G hi, C lo, G lo}, entry 3 c + k for part c
// and factor k (eresp_coef_kernel; frame_step_n, frame_block_end_n below
// generalise the step to cubic parts).  W = y_W in every frame, so the
// remainder's source reads its accumulator directly.  The rounding: 2^-48 of
// the accumulator per double-FP32 addition over one block's ~150 additions
// (~5e-14 of the parts' terms), the rest FP64.
constexpr int kStateRow = 9;
constexpr int kFrameSmemRows = 112;  // rows staged in shared memory (15.75 KB per CTA at most)

// fn(std::integral_constant<int, G>) for the groups G = ceil(n_act/4) - 1 .. 0
// of four slots each, by a switch that enters a fall-through chain (Duff's
// device): no instruction of a skipped group issues, and each group is one
// basic block (its loads in flight together, its chains interleaved).
template <typename Fn>
__device__ __forceinline__ void resp_groups(int n_act, Fn&& fn)
{
    static_assert(kRespSlots == 24, "six groups of four slots");
    switch ((n_act + 3) >> 2) {
        case 6:
            fn(std::integral_constant<int, 5>{});
            [[fallthrough]];
        case 5:
            fn(std::integral_constant<int, 4>{});
            [[fallthrough]];
        case 4:
            fn(std::integral_constant<int, 3>{});
            [[fallthrough]];
        case 3:
            fn(std::integral_constant<int, 2>{});
            [[fallthrough]];
        case 2:
            fn(std::integral_constant<int, 1>{});
            [[fallthrough]];
        case 1:
            fn(std::integral_constant<int, 0>{});
            [[fallthrough]];
        default:
            break;
    }
}

// resp_groups with the step's other work, tail(), in one basic block with
// the last M groups (groups M-1 .. 0; all active groups when fewer are): the
// tail's instructions and those groups' chains interleave instead of
// following one another.  Groups above them keep their own blocks.
template <int M, typename Fn, typename Tail>
__device__ __forceinline__ void resp_groups_tail(int n_act, Fn&& fn, Tail&& tail)
{
    static_assert(kRespSlots == 24 && M >= 1 && M <= 3, "six groups of four slots; 1 to 3 merged");
    using I0 = std::integral_constant<int, 0>;
    using I1 = std::integral_constant<int, 1>;
    using I2 = std::integral_constant<int, 2>;
    switch ((n_act + 3) >> 2) {
        case 6:
            fn(std::integral_constant<int, 5>{});
            [[fallthrough]];
        case 5:
            fn(std::integral_constant<int, 4>{});
            [[fallthrough]];
        case 4:
            fn(std::integral_constant<int, 3>{});
            [[fallthrough]];
        case 3:
            fn(I2{});
            if constexpr (M >= 3) {
                fn(I1{});
                fn(I0{});
                tail();
                break;
            }
            [[fallthrough]];
        case 2:
            fn(I1{});
            if constexpr (M >= 2) {
                fn(I0{});
                tail();
                break;
            }
            [[fallthrough]];
        case 1:
            fn(I0{});
            tail();
            break;
        default:
            tail();
            break;
    }
}

}  // namespace hjm

namespace hjm {

// ---------------------------------------------------------------------------
// The polynomial parts with NP = 3 or 4 components (degree <= 3), for the
// generalised Euler response kernel (hjm_eresp.cu).  The parts are the
// coefficients x_d of the stochastic curve's polynomial sum_d x_d t^d in
// t = T - tau0 (tau0 = 0 for the quadratic forms, the last tenor T_L for the
// cubic one).  The upwind step takes t^d to t^d + c ((t + dtau)^d - t^d) at
// every tenor below L (a translation, so the centre does not matter), i.e.
// x <- M x + B phi with M = I + N,
//     N[i][d] = c C(d, i) dtau^(d - i)   (i < d):
//     n01 = c dtau, n02 = c dtau^2, n03 = c dtau^3, n12 = 2 c dtau,
//     n13 = 3 c dtau^2, n23 = 3 c dtau,
// and at L, where the scheme takes the backward difference, the polynomial
// is off by -c (P(T_L + dtau) - 2 P(T_L) + P(T_L - dtau)) e_L: the remainder's
// source.  With tau0 = T_L that second difference vanishes for t^3 (and for
// 1, t), so the source stays -2 c dtau^2 x_2 e_L, one term in W = x_2.
// N is nilpotent (N^NP = 0), so every power series in N is a cubic in N:
//     M^a   = sum_i C(a, i) N^i,
//     M^-k  = sum_i (-1)^i C(k + i - 1, i) N^i,
//     Q(a)  = sum_{e=1..a} M^e = a I + sum_{i>=1} C(a + 1, i + 1) N^i.
// A matrix c0 I + c1 N + c2 N^2 + c3 N^3 has the entries of PolyN below.
// ---------------------------------------------------------------------------
struct PartsN {
    double n01, n02, n03, n12, n13, n23;
};

// Entries of c0 I + c1 N + c2 N^2 + c3 N^3 above the diagonal (the diagonal is c0).
struct PolyN {
    double d, e01, e02, e03, e12, e13, e23;
    __host__ __device__ PolyN() : d(0), e01(0), e02(0), e03(0), e12(0), e13(0), e23(0) {}
    __host__ __device__ PolyN(const PartsN& n, double c0, double c1, double c2, double c3)
    {
        d = c0;
        e01 = c1 * n.n01;
        e12 = c1 * n.n12;
        e23 = c1 * n.n23;
        e02 = c1 * n.n02 + c2 * (n.n01 * n.n12);
        e13 = c1 * n.n13 + c2 * (n.n12 * n.n23);
        e03 = c1 * n.n03 + c2 * (n.n01 * n.n13 + n.n02 * n.n23) + c3 * (n.n01 * n.n12 * n.n23);
    }
    // row r of the matrix times x (NP = 4 entries, unused ones zero)
    __host__ __device__ double row(int r, const double* x) const
    {
        switch (r) {
            case 0: return d * x[0] + e01 * x[1] + e02 * x[2] + e03 * x[3];
            case 1: return d * x[1] + e12 * x[2] + e13 * x[3];
            case 2: return d * x[2] + e23 * x[3];
            default: return d * x[3];
        }
    }
};

// M^a and Q(a) of a block of a steps, FP64, formed once on the host.
struct BlockFrameN {
    PolyN Ma, Qa;
};

inline double binom(double a, int i)
{
    double r = 1.0;
    for (int j = 0; j < i; ++j) r = r * (a - j) / (double)(j + 1);
    return r;
}

inline BlockFrameN block_frame_n(const PartsN& n, int a)
{
    const double da = (double)a;
    BlockFrameN f;
    f.Ma = PolyN(n, 1.0, binom(da, 1), binom(da, 2), binom(da, 3));
    f.Qa = PolyN(n, da, binom(da + 1.0, 2), binom(da + 1.0, 3), binom(da + 1.0, 4));
    return f;
}

// The degrees of the three factors packed in one template constant.
__host__ __device__ constexpr int degs_pack(int d0, int d1, int d2) { return d0 | (d1 << 2) | (d2 << 4); }
__host__ __device__ constexpr int degs_of(int pack, int k) { return (pack >> (2 * k)) & 3; }
__host__ __device__ constexpr int degs_parts(int pack)
{
    return 1 + (degs_of(pack, 0) > degs_of(pack, 1) ? (degs_of(pack, 0) > degs_of(pack, 2) ? degs_of(pack, 0)
                                                                                          : degs_of(pack, 2))
                                                    : (degs_of(pack, 1) > degs_of(pack, 2) ? degs_of(pack, 1)
                                                                                          : degs_of(pack, 2)));
}
// Coefficient-row length of NP parts: entry 3 c + k for part c and factor k,
// then (NP = 4) the source coefficient s n23 of the step.
__host__ __device__ constexpr int frame_row(int np) { return np == 4 ? 13 : 9; }

// One step of the NP parts in the moving frame: y_c += C(s)[c][k] phi_k and
// v_c += G(s)[c][k] phi_k for the terms (c, k) with c <= deg_k (part c of
// M^-(s+1) B is zero for factors of lower degree), each part renormalised
// after its last term.  cr: the step's coefficient row (shared memory or L1).
template <int DEGS, bool EXT, bool SHARED>
__device__ __forceinline__ void frame_step_n(float2 (&Y)[degs_parts(DEGS)], float2 (&Yl)[degs_parts(DEGS)],
                                             const float4* __restrict__ cr, const float (&ph)[3],
                                             const float (&pl)[3])
{
    constexpr int NP = degs_parts(DEGS);
    float4 q[3 * NP];
#pragma unroll
    for (int t = 0; t < 3 * NP; ++t)
        if (t / 3 <= degs_of(DEGS, t % 3)) {
            if constexpr (SHARED)
                q[t] = cr[t];
            else
                q[t] = __ldg(cr + t);
        }
#pragma unroll
    for (int c = 0; c < NP; ++c) {
#pragma unroll
        for (int k = 0; k < 3; ++k) {
            if (c > degs_of(DEGS, k)) continue;
            const float4 e = q[3 * c + k];
            const float2 kh = make_float2(e.x, e.y), kl = make_float2(e.z, e.w);
            if constexpr (EXT)
                df_acc(Y[c], Yl[c], kh, kl, make_float2(ph[k], ph[k]), make_float2(pl[k], pl[k]),
                       make_float2(-ph[k], -ph[k]));
            else
                df_acc_w(Y[c], Yl[c], kh, kl, make_float2(ph[k], ph[k]), make_float2(-ph[k], -ph[k]));
        }
        df_renorm(Y[c], Yl[c]);
    }
}

// The end of a block of the NP parts: x = M^a y, Z += Q(a) y - v (z[c *
// stride_z], FP64 in shared memory), then y re-anchored on x (v = 0).
template <int NP>
__device__ __forceinline__ void frame_block_end_n(float2 (&Y)[NP], float2 (&Yl)[NP], const BlockFrameN& F, double* z,
                                                  int stride_z, double (&x)[NP], double (&Z)[NP])
{
    double y[4] = {0.0, 0.0, 0.0, 0.0}, v[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int c = 0; c < NP; ++c) {
        y[c] = widen_f32(Y[c].x) + widen_f32(Yl[c].x);
        v[c] = widen_f32(Y[c].y) + widen_f32(Yl[c].y);
    }
#pragma unroll
    for (int c = 0; c < NP; ++c) {
        x[c] = F.Ma.row(c, y);
        Z[c] = z[c * stride_z] + (F.Qa.row(c, y) - v[c]);
        z[c * stride_z] = Z[c];
    }
#pragma unroll
    for (int c = 0; c < NP; ++c) {
        const float xh = __double2float_rn(x[c]);
        Y[c] = make_float2(xh, 0.0f);
        Yl[c] = make_float2(__double2float_rn(x[c] - (double)xh), 0.0f);
    }
}

}  // namespace hjm
