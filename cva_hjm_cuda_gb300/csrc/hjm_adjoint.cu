// hjm_adjoint.cu -- pathwise adjoint of the CVA (one fused launch per path tile).
//
// New work: the reference lists AAD / pathwise sensitivities as to-do items
// (doc/TODO:6,14) and computes none.  Per path the kernel runs the mixed
// precision forward valuation of hjm_forward.cu (FP32 curve and pricing, FP64
// discount sums), then a reverse sweep over the Euler steps, and reduces the
// path's contributions to dCVA/d(initial forwards), dCVA/d(drift table) and
// dCVA/d(polynomial volatility coefficients) inside the CTA.
//
// Adjoint algebra.  With f = p + h (deterministic + stochastic part) and the
// Euler map f_n = A f_{n-1} + dt mu + S phi_n (A: the constant upwind
// convection operator, S[t][k] = sqrt(dt) sigma_k(tau_t)), the adjoint of the
// state obeys
//     g_{n-1} = A^T g_n + seeds_{n-1},
// where the seeds come from the pricing: tenor i is read as the forward x_i at
// step n_i = stride*i - 1 and as the discount sum a_i = sum_{n <= n_i} f_n[i],
// so seeds_n[i] = abar_i for n <= n_i and xbar_i at n = n_i, with
//     cfbar_i = sum_{j<i} w_j [V_j > 0],  V_j = sum_{i>j} cf_i,
//     xbar_i = cfbar_i D_i payA_i e^{x_i/m},  abar_i = -dt D_i cfbar_i (payA_i L_i - payB_i).
// The Jacobian A does not depend on the state.  Two consequences shape the kernel:
//  * h does not depend on the initial curve or the drift, so dCVA/dspot and
//    dCVA/dmu follow from the path means of the per-date seeds (E xbar_i,
//    E abar_i) through the adjoint of the deterministic curve p, which the host
//    runs in FP64; the kernel only reduces those 2B means.
//  * the volatility coefficients (sigma_k(T) = sum_d c_{k,d} T^d) need, per step,
//    the three moments M_d(n) = sum_t g_n[t] tau_t^d:
//        dCVA/dc_{k,d} (diffusion) = sqrt(dt) sum_n phi_{n,k} M_d(n),
//    and because A 1 = 1, A tau = tau + c dtau 1 and A tau^2 = tau^2 + 2 c dtau tau
//    + c dtau^2 1 - 2 c dtau^2 e_L, the moments of A^T g follow from those of g
//    and g[L] in O(1):  M0' = M0,  M1' = M1 + c dtau M0,
//        M2' = M2 + 2 c dtau M1 + c dtau^2 M0 - 2 c dtau^2 g[L].
//    The per-tenor state g is still swept (A^T on packed pairs) for g[L].
// The drift's own dependence on the coefficients (trapezoid rule) is chained
// on the host.  The normals are regenerated from their Philox counters.
//
// Checkpoint mode (checkpoint_every = K in [1, stride]).  The forward pass
// keeps only the cash flows; before every K-th Euler step whose segment holds
// a date's sampling step it writes the path's state (scaled curve, polynomial
// parts, scales) and the FP64 discount sum of the next tenor to be sampled to
// HBM.  Because the Jacobian is state-independent, the reverse sweep needs the
// forward state only at the sampling steps: the seed pass recomputes each
// date's state from the last checkpoint before it (at most K steps, repeating
// the forward arithmetic from the stored state) and forms the date's seeds;
// the sweep then runs backwards over the steps with the regenerated normals.
// With K = 0 the forward pass keeps the per-date (x_i, D_i) instead and
// nothing is recomputed.
#include <cuda_runtime.h>

#include <cstdint>

#include "hjm_device.cuh"
#include "hjm_kernels.h"
#include "hjm_pairs.cuh"
#include "hjm_pc.cuh"

namespace hjm {

constexpr int kAdjCta = 64;  // paths per CTA of the adjoint kernel

// Shared memory per thread (thread-private columns, stride kAdjCta):
//   acc_s  (B+1) f64   FP64 discount sums, slot i then cash flow i
//   hs_s   (B+2) f32   curve at the block start (forward), exposures (forward
//                      epilogue), curve at the segment start (recompute)
//   xs_s   (B+1) f32   K = 0: x_i then xbar_i;  K > 0: cfbar_i then xbar_i
//   ds_s   (B+1) f32   K = 0: D_i then abar_i;   K > 0: abar_i
//   cb_s   9 f64       diffusion coefficient adjoints
//   red_s  (kAdjCta/32) * R f64   CTA reduction
// With checkpoints (K > 0) xs_s and ds_s are first written after the
// exposures have consumed the cash flows (a barrier between), so they take
// acc_s's place: a third less shared memory per CTA, which sets the
// occupancy when there are many dates.
struct AdjLayout {
    size_t acc, hs, xs, ds, cb, red, total;
};

__host__ __device__ inline size_t align128(size_t x) { return (x + 127) & ~(size_t)127; }

__host__ __device__ inline AdjLayout adj_layout(int nt, int B, int R, bool ckpt = false)
{
    AdjLayout L;
    (void)nt;
    const size_t rows = (size_t)B + 1;
    L.acc = 0;
    L.hs = align128(rows * 8 * kAdjCta);
    if (ckpt) {
        L.xs = L.acc;
        L.ds = L.acc + rows * kAdjCta * 4;
        L.cb = align128(L.hs + (rows + 1) * kAdjCta * 4);
    } else {
        L.xs = align128(L.hs + (rows + 1) * kAdjCta * 4);
        L.ds = align128(L.xs + rows * kAdjCta * 4);
        L.cb = align128(L.ds + rows * kAdjCta * 4);
    }
    L.red = align128(L.cb + (size_t)9 * kAdjCta * 8);
    L.total = align128(L.red + (size_t)(kAdjCta / 32) * R * 8);
    return L;
}

// Seeds of date i from its sampled forward x, discount factor D and cfbar.
__device__ __forceinline__ void date_seeds(const PathParams<float>& P, int i, double x, float D, float cfbar,
                                           float& xbar, float& abar)
{
    const float mm = (float)P.m;
    const float xf = (float)x;
    const float e = expf(xf / mm);
    const float L = mm * expm1f(xf / mm);
    const float pa = (float)P.payA[i], pbk = (float)P.payB[i];
    xbar = cfbar * D * pa * e;
    abar = -(float)P.dt * D * cfbar * (pa * L - pbk);
}

template <int NT>
__device__ __forceinline__ void pair_set(float2 (&v)[PairGrid<NT>::H], int i, float val)
{
    constexpr int H = PairGrid<NT>::H;
#pragma unroll
    for (int p = 0; p < H; ++p) {
        if (p == i) v[p].x = val;
        if (p + H == i) v[p].y = val;
    }
}

template <int NT>
__device__ __forceinline__ void pair_add(float2 (&v)[PairGrid<NT>::H], int i, float val)
{
    constexpr int H = PairGrid<NT>::H;
#pragma unroll
    for (int p = 0; p < H; ++p) {
        if (p == i) v[p].x += val;
        if (p + H == i) v[p].y += val;
    }
}

// Resident CTAs per SM: the reverse sweep holds 2 ceil(NT/2) float2 (adjoint
// state and discount seeds) besides the normals' state.  Registers are
// granted per scheduler (16 K each), so 6 CTAs of 2 warps (3 warps per
// scheduler, 168 registers) is the budget for 51 tenors and 4 CTAs (2 warps
// per scheduler, 255 registers) keeps 61 tenors free of spills.
template <int NT>
constexpr int adj_min_ctas() { return NT > 56 ? 4 : 6; }

template <int NT, bool CKPT, bool POLY>
__global__ void __launch_bounds__(kAdjCta, adj_min_ctas<NT>())
    adjoint_kernel(const __grid_constant__ AdjParams A, double* __restrict__ partials, float* __restrict__ ck_h,
                   double* __restrict__ ck_a)
{
    constexpr int H = PairGrid<NT>::H;
    constexpr int kCtaA = kAdjCta;
    const MixedParams& M = A.M;
    const PathParams<float>& P = M.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const int rows = B + 1;
    const int R = 3 * B + 12;
    const AdjLayout Ly = adj_layout(NT, B, R, CKPT);
    double* acc_s = reinterpret_cast<double*>(smem + Ly.acc);
    float* hs_s = reinterpret_cast<float*>(smem + Ly.hs);
    float* xs_s = reinterpret_cast<float*>(smem + Ly.xs);
    float* ds_s = reinterpret_cast<float*>(smem + Ly.ds);
    double* cb_s = reinterpret_cast<double*>(smem + Ly.cb);
    double* red_s = reinterpret_cast<double*>(smem + Ly.red);

    const int64_t lp = (int64_t)blockIdx.x * kCtaA + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;
    const int stride = P.stride;
    const int n_steps = B * stride;
    const int K = CKPT ? A.ckpt_every : stride;
    const int64_t ld = A.ck_ld;

    // ---------------------------------------------------------------- forward
    // The same arithmetic as path_kernel_mixed, plus what the sweep needs.
    MixedPath<NT, POLY> x;
    x.reset();
    for (int i = 0; i < rows; ++i) acc_s[i * kCtaA + tid] = 0.0;
    for (int t = 0; t <= B + 1; ++t) hs_s[t * kCtaA + tid] = 0.f;

    auto sample = [&](int i) {
        const double xv = P.psamp[i] + (double)x.value(P, i);
        const double a = P.psum[i] + acc_s[i * kCtaA + tid];
        const float D = expf((float)(-a * P.dt));
        const float mm = (float)P.m;
        const float L = mm * expm1f((float)xv / mm);
        acc_s[i * kCtaA + tid] = (double)(D * ((float)P.payA[i] * L - (float)P.payB[i]));
        if (!CKPT) {
            xs_s[i * kCtaA + tid] = (float)xv;
            ds_s[i * kCtaA + tid] = D;
        }
    };

    // checkpoint rows: the NT tenors of the scaled curve v (POLY: its convected
    // part), then S, U, W and the scales g, ig: the recomputation restarts from
    // the forward pass's own state and repeats its arithmetic
    constexpr int kCkRows = NT + 5;
    sample(1);
    int ck = 0, ck_next = stride;  // next checkpoint: before step ck_next
    const int n_last = n_steps - 1;
    float q0, q1, q2;  // normals drawn one step ahead (as in path_kernel_mixed)
    draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, stride, P.rk0, P.rk1, q0, q1, q2);
    for (int b = 1; b < B; ++b) {
        BlockSums bs;
        bs.reset();
        x.begin_block(P, b);
        for (int s = 0; s < stride; ++s) {
            const int n = b * stride + s;
            if (CKPT && n == ck_next) {
                // checkpoint before step n: the curve, and the discount sum of the
                // next tenor to be sampled (completed blocks + this block so far,
                // the latter recovered from the partial sums of the block)
                ck_next += K;
                const int inext = b + 1;
                // only a segment that holds a date's sampling step (the block's
                // last step) is ever restarted by the seed pass
                const bool needed = (b + 1) * stride - 1 < n + K;
                double part = 0.0;
                if (needed && s > 0)
                    block_sums_up<NT, POLY>(x, hs_s, tid, kCtaA, P, bs, inext, [&](int t, float Ht) {
                        if (t == inext) part = as_f64(Ht);
                    });
                if (needed && active) {
#pragma unroll
                    for (int t = 0; t < NT; ++t) ck_h[((size_t)ck * kCkRows + t) * ld + lp] = pair_tenor<NT>(x.h, t);
                    ck_h[((size_t)ck * kCkRows + NT) * ld + lp] = x.S;
                    ck_h[((size_t)ck * kCkRows + NT + 1) * ld + lp] = x.U;
                    ck_h[((size_t)ck * kCkRows + NT + 2) * ld + lp] = x.W;
                    ck_h[((size_t)ck * kCkRows + NT + 3) * ld + lp] = x.g;
                    ck_h[((size_t)ck * kCkRows + NT + 4) * ld + lp] = x.ig;
                    ck_a[(size_t)ck * ld + lp] = acc_s[inext * kCtaA + tid] + part;
                }
                ++ck;
            }
            const float phi0 = q0, phi1 = q1, phi2 = q2;
            draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, min(n + 1, n_last), P.rk0, P.rk1, q0, q1, q2);
            x.step(M, phi0, phi1, phi2);
            bs.add(x, phi0, phi1, phi2);
        }
        block_sums_up<NT, POLY>(x, hs_s, tid, kCtaA, P, bs, B, [&](int t, float Ht) {
            if (t > b) acc_s[t * kCtaA + tid] += as_f64(Ht);
        });
#pragma unroll
        for (int t = 1; t < NT; ++t)
            if (t <= B + 1) hs_s[t * kCtaA + tid] = x.rem(t);
        sample(b + 1);
    }

    // exposures, the path's CVA contribution, the CTA's EE and CVA partial sums
    float* e_s = hs_s;
    double v = 0.0, cva_c = 0.0;
    e_s[B * kCtaA + tid] = 0.f;
    for (int j = B - 1; j >= 0; --j) {
        v += acc_s[(j + 1) * kCtaA + tid];
        double e = (v > 0.0) ? v : 0.0;
        if (!active) e = 0.0;
        e_s[j * kCtaA + tid] = (float)e;
        cva_c = fma(P.cvaw[j], e, cva_c);
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    for (int j = warp; j <= B; j += kCtaA / 32) {
        double sum = 0.0;
#pragma unroll
        for (int q = 0; q < kCtaA / 32; ++q) sum += (double)e_s[j * kCtaA + lane + 32 * q];
        sum = warp_sum(sum);
        if (lane == 0) partials[(size_t)blockIdx.x * R + j] = sum;
    }
    {
        const double s1 = warp_sum(cva_c), s2 = warp_sum(cva_c * cva_c);
        if (lane == 0) {
            red_s[warp] = s1;
            red_s[kCtaA / 32 + warp] = s2;
        }
    }
    __syncthreads();
    if (tid == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kCtaA / 32; ++w) {
            s1 += red_s[w];
            s2 += red_s[kCtaA / 32 + w];
        }
        partials[(size_t)blockIdx.x * R + B + 1] = s1;
        partials[(size_t)blockIdx.x * R + B + 2] = s2;
    }

    // cfbar_i = sum_{j<i} w_j [E_j > 0]; per-date seeds (K = 0) or cfbar kept (K > 0)
    {
        float cfbar = 0.f;
        for (int i = 1; i <= B; ++i) {
            const int j = i - 1;
            if (e_s[j * kCtaA + tid] > 0.f) cfbar += (float)P.cvaw[j];
            if (!active) cfbar = 0.f;
            if (CKPT) {
                xs_s[i * kCtaA + tid] = cfbar;
            } else {
                float xbar, abar;
                date_seeds(P, i, (double)xs_s[i * kCtaA + tid], ds_s[i * kCtaA + tid], cfbar, xbar, abar);
                xs_s[i * kCtaA + tid] = xbar;
                ds_s[i * kCtaA + tid] = abar;
            }
        }
    }

    // ------------------------------------------------- date seeds (checkpoints)
    // The sweep needs the forward state only where the pricing reads it: the
    // sampled forward and discount of each date.  Each date's state is
    // recomputed from the last checkpoint before its sampling step (at most K
    // steps, inside one block), repeating the forward pass's arithmetic from
    // its stored state; date 1 is deterministic (h = 0 through block 0).
    if (CKPT) {
        for (int i = B; i >= 1; --i) {
            float xb, ab;
            if (i == 1) {
                const float D1 = expf((float)(-P.psum[1] * P.dt));
                date_seeds(P, 1, P.psamp[1], D1, xs_s[1 * kCtaA + tid], xb, ab);
            } else {
                const int ni = i * stride - 1;   // the step that samples date i
                const int sg = (ni - stride) / K;
                const int n0 = stride + sg * K;  // its checkpoint
                MixedPath<NT, POLY> xr;
                const size_t base = (size_t)sg * kCkRows;
#pragma unroll
                for (int p = 0; p < H; ++p) {
                    xr.h[p].x = active ? ck_h[(base + p) * ld + lp] : 0.f;
                    xr.h[p].y = (active && p + H < NT) ? ck_h[(base + p + H) * ld + lp] : 0.f;
                }
                xr.S = active ? ck_h[(base + NT) * ld + lp] : 0.f;
                xr.U = active ? ck_h[(base + NT + 1) * ld + lp] : 0.f;
                xr.W = active ? ck_h[(base + NT + 2) * ld + lp] : 0.f;
                xr.g = active ? ck_h[(base + NT + 3) * ld + lp] : 1.f;
                xr.ig = active ? ck_h[(base + NT + 4) * ld + lp] : 1.f;
#pragma unroll
                for (int t = 1; t < NT; ++t)
                    if (t <= B + 1) hs_s[t * kCtaA + tid] = xr.rem(t);
                const double a0 = active ? ck_a[(size_t)sg * ld + lp] : 0.0;
                BlockSums bs;
                bs.reset();
                float r0, r1, r2;
                draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, n0, P.rk0, P.rk1, r0, r1, r2);
                for (int n = n0; n <= ni; ++n) {
                    const float phi0 = r0, phi1 = r1, phi2 = r2;
                    draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, min(n + 1, ni), P.rk0, P.rk1, r0, r1, r2);
                    xr.step(M, phi0, phi1, phi2);
                    bs.add(xr, phi0, phi1, phi2);
                }
                double part = 0.0;
                block_sums_up<NT, POLY>(xr, hs_s, tid, kCtaA, P, bs, i, [&](int t, float Ht) {
                    if (t == i) part = as_f64(Ht);
                });
                const double xv = P.psamp[i] + (double)xr.value(P, i);
                const double a = P.psum[i] + a0 + part;
                const float D = expf((float)(-a * P.dt));
                date_seeds(P, i, xv, D, xs_s[i * kCtaA + tid], xb, ab);
            }
            xs_s[i * kCtaA + tid] = xb;  // the seeds replace cfbar (no longer needed)
            ds_s[i * kCtaA + tid] = ab;
        }
    }

    // ---------------------------------------------------------------- reverse
    for (int q = 0; q < 9; ++q) cb_s[q * kCtaA + tid] = 0.0;
    float2 g[H], inj[H];
#pragma unroll
    for (int p = 0; p < H; ++p) {
        g[p] = make_float2(0.f, 0.f);
        inj[p] = make_float2(0.f, 0.f);
    }
    // moments of g and of the injected discount seeds
    float M0 = 0.f, M1 = 0.f, M2 = 0.f, I0 = 0.f, I1 = 0.f, I2 = 0.f;
    const float dtau = (float)(1.0 / P.m);
    const float k1 = P.c * dtau, k2 = P.c * dtau * dtau;

    // block i-1 (steps (i-1) stride .. i stride - 1) ends by sampling date i;
    // normals drawn one step ahead (descending)
    float r0, r1, r2;
    draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, n_steps - 1, P.rk0, P.rk1, r0, r1, r2);
    for (int i = B; i >= 2; --i) {
        {
            // date i: its discount seed switches on for all earlier steps, its
            // forward seed enters at its sampling step
            const float xb = xs_s[i * kCtaA + tid], ab = ds_s[i * kCtaA + tid];
            pair_set<NT>(inj, i, ab);
            pair_add<NT>(g, i, xb);
            const float ti = dtau * (float)i;
            I0 += ab;
            I1 = fmaf(ab, ti, I1);
            I2 = fmaf(ab, ti * ti, I2);
            M0 += xb;
            M1 = fmaf(xb, ti, M1);
            M2 = fmaf(xb, ti * ti, M2);
        }
        float cbb[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) cbb[q] = 0.f;
        // g holds the adjoint times (1 + rr)^k after k steps of this block
        float sig = 1.f, gam = 1.f;  // (1 + rr)^k and its inverse
        for (int n = i * stride - 1; n >= (i - 1) * stride; --n) {
            M0 += I0;
            M1 += I1;
            M2 += I2;
            const float phi0 = r0, phi1 = r1, phi2 = r2;
            draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, max(n - 1, stride), P.rk0, P.rk1, r0, r1, r2);
            cbb[0] = fmaf(phi0, M0, cbb[0]);
            cbb[1] = fmaf(phi0, M1, cbb[1]);
            cbb[2] = fmaf(phi0, M2, cbb[2]);
            cbb[3] = fmaf(phi1, M0, cbb[3]);
            cbb[4] = fmaf(phi1, M1, cbb[4]);
            cbb[5] = fmaf(phi1, M2, cbb[5]);
            cbb[6] = fmaf(phi2, M0, cbb[6]);
            cbb[7] = fmaf(phi2, M1, cbb[7]);
            cbb[8] = fmaf(phi2, M2, cbb[8]);
            // the sweep itself (seeds of this step folded in), then the
            // moments of A^T g from those of g and its last tenor
            float GL;
            adjoint_step_pairs<NT>(g, inj, sig, P.rr, GL);
            const float gL = gam * GL;
            M2 = fmaf(-2.f * k2, gL, fmaf(k2, M0, fmaf(2.f * k1, M1, M2)));
            M1 = fmaf(k1, M0, M1);
            sig *= P.ip;
            gam *= P.qm;
        }
        {
            const float2 gg = make_float2(gam, gam);
#pragma unroll
            for (int p = 0; p < H; ++p) g[p] = __fmul2_rn(g[p], gg);
        }
        // fold the block's FP32 partials
#pragma unroll
        for (int q = 0; q < 9; ++q) cb_s[q * kCtaA + tid] += (double)cbb[q];
    }

    // ---------------------------------------------------------------- CTA reduction
    // columns: [0..B] EE, B+1/B+2 CVA stats (written above), then
    // E xbar_i (i = 1..B), E abar_i (i = 1..B), and the 9 coefficient columns
    const int cx = B + 3, ca = 2 * B + 3, cc = 3 * B + 3;
    double* wred = red_s;  // [warp][R]
    for (int i = 1; i <= B; ++i) {
        const double sx_ = warp_sum(active ? (double)xs_s[i * kCtaA + tid] : 0.0);
        const double sa_ = warp_sum(active ? (double)ds_s[i * kCtaA + tid] : 0.0);
        if (lane == 0) {
            wred[warp * R + cx + i - 1] = sx_;
            wred[warp * R + ca + i - 1] = sa_;
        }
    }
    for (int q = 0; q < 9; ++q) {
        const double sum = warp_sum(active ? cb_s[q * kCtaA + tid] : 0.0);
        if (lane == 0) wred[warp * R + cc + q] = sum;
    }
    __syncthreads();
    for (int col = cx + tid; col < R; col += kCtaA) {
        double sum = 0.0;
        for (int w = 0; w < kCtaA / 32; ++w) sum += wred[w * R + col];
        partials[(size_t)blockIdx.x * R + col] = sum;
    }
}

// ---------------------------------------------------------------------------
// Predictor-corrector adjoint (mixed precision; the sampled states are kept,
// checkpoint_every = 0).  The forward pass is the valuation's (PcPath: FP32
// curve with the effective scheme a0e, a1e, a2e and Euler rows with ce at
// L-1, L; FP64 discount sums), so the CVA equals the predictor-corrector
// valuation's bit for bit.  The reverse sweep carries the per-tenor adjoint
// through the transpose of that scheme,
//     (A2^T v)[t] = a0e v[t] + a1e v[t-1] + a2e v[t-2]                 (t <= L-2),
//     (A2^T v)[L-1] = a1e v[L-2] + a2e v[L-3] + (1 - ce) v[L-1] - ce v[L],
//     (A2^T v)[L]   = a2e v[L-2] + ce v[L-1] + (1 + ce) v[L],
// and the moments M_d = sum_t g[t] tau_t^d through A2's action on the
// polynomial basis (the forward's decomposition constants):
//     M1' = M1 + c dtau M0,  M2' = M2 + 2 c dtau M1 + (c + c^2) dtau^2 M0 + wL1 g[L-1] + wL g[L].
// The noise enters through the N-projected loadings alpha = aS.phi (S), beta
// = aU.phi (U), gamma = aW.phi (W, and gL gamma at the last tenor), so per
// step the coefficient columns gather phi_k (M0, M1, M2 + gL g[L]); the host
// chains them to the coefficients (aS, aU, aW are linear in them) and runs
// the FP64 adjoint of the deterministic curve p' = A2 p + N mu dt.
struct PcAdjLayout {
    size_t acc, hs, xs, ds, cb, red, total;
};

__host__ __device__ inline PcAdjLayout pc_adj_layout(int nt, int B, int R)
{
    PcAdjLayout L;
    const size_t rows = (size_t)B + 1;
    const size_t hs_rows = (size_t)(nt > B + 1 ? nt : B + 1);
    L.acc = 0;
    L.hs = align128(rows * 8 * kPcCta);
    L.xs = align128(L.hs + hs_rows * kPcCta * 4);
    L.ds = align128(L.xs + rows * kPcCta * 4);
    L.cb = align128(L.ds + rows * kPcCta * 4);
    L.red = align128(L.cb + (size_t)9 * kPcCta * 8);
    L.total = align128(L.red + (size_t)(kPcCta / 32) * R * 8);
    return L;
}

template <int NT, bool POLY>
__global__ void __launch_bounds__(kPcCta, 4)
    adjoint_kernel_pc(const __grid_constant__ PcParams<float> Q, double* __restrict__ partials)
{
    constexpr int L = NT - 1;
    constexpr int kC = kPcCta;
    const PathParams<float>& P = Q.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const int R = 3 * B + 12;
    const PcAdjLayout Ly = pc_adj_layout(NT, B, R);
    double* acc_s = reinterpret_cast<double*>(smem + Ly.acc);
    float* hs_s = reinterpret_cast<float*>(smem + Ly.hs);
    float* xs_s = reinterpret_cast<float*>(smem + Ly.xs);
    float* ds_s = reinterpret_cast<float*>(smem + Ly.ds);
    double* cb_s = reinterpret_cast<double*>(smem + Ly.cb);
    double* red_s = reinterpret_cast<double*>(smem + Ly.red);

    const int64_t lp = (int64_t)blockIdx.x * kC + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;
    const int stride = P.stride;
    const int n_steps = B * stride;

    // ---------------------------------------------------------------- forward
    PcPath<NT, float, POLY> x;
    x.reset();
    for (int i = 0; i <= B; ++i) acc_s[i * kC + tid] = 0.0;
    for (int t = 0; t < NT; ++t) hs_s[t * kC + tid] = 0.f;
    auto sample = [&](int i) {
        const double xv = P.psamp[i] + (double)x.value(P, i);
        const double a = P.psum[i] + acc_s[i * kC + tid];
        const float D = exp_t<float>((float)(-a * P.dt));
        const float mm = (float)P.m;
        const float Lb = mm * expm1_t<float>((float)xv / mm);
        acc_s[i * kC + tid] = (double)(D * ((float)P.payA[i] * Lb - (float)P.payB[i]));
        xs_s[i * kC + tid] = (float)xv;
        ds_s[i * kC + tid] = D;
    };
    sample(1);
    for (int b = 1; b < B; ++b) {
        x.begin_block(P, b);
        for (int s = 0; s < stride; ++s) {
            float phi0, phi1, phi2;
            draw_phi<float, false>(nullptr, gpath, active ? lp : 0, P.n_paths, b * stride + s, P.rk0, P.rk1, phi0,
                                   phi1, phi2);
            x.step(Q, phi0, phi1, phi2);
        }
        x.end_block(Q, b, B, hs_s, acc_s, tid);
        sample(b + 1);
    }

    // exposures, the path's CVA contribution, the CTA's EE and CVA partial sums
    float* e_s = hs_s;
    double vsum = 0.0, cva_c = 0.0;
    e_s[B * kC + tid] = 0.f;
    for (int j = B - 1; j >= 0; --j) {
        vsum += acc_s[(j + 1) * kC + tid];
        double e = (vsum > 0.0) ? vsum : 0.0;
        if (!active) e = 0.0;
        e_s[j * kC + tid] = (float)e;
        cva_c = fma(P.cvaw[j], e, cva_c);
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    for (int j = warp; j <= B; j += kC / 32) {
        double sum = 0.0;
#pragma unroll
        for (int q = 0; q < kC / 32; ++q) sum += (double)e_s[j * kC + lane + 32 * q];
        sum = warp_sum(sum);
        if (lane == 0) partials[(size_t)blockIdx.x * R + j] = sum;
    }
    {
        const double s1 = warp_sum(cva_c), s2 = warp_sum(cva_c * cva_c);
        if (lane == 0) {
            red_s[warp] = s1;
            red_s[kC / 32 + warp] = s2;
        }
    }
    __syncthreads();
    if (tid == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kC / 32; ++w) {
            s1 += red_s[w];
            s2 += red_s[kC / 32 + w];
        }
        partials[(size_t)blockIdx.x * R + B + 1] = s1;
        partials[(size_t)blockIdx.x * R + B + 2] = s2;
    }
    // per-date seeds from cfbar_i = sum_{j<i} w_j [E_j > 0]
    {
        float cfbar = 0.f;
        for (int i = 1; i <= B; ++i) {
            if (e_s[(i - 1) * kC + tid] > 0.f) cfbar += (float)P.cvaw[i - 1];
            if (!active) cfbar = 0.f;
            float xbar, abar;
            date_seeds(P, i, (double)xs_s[i * kC + tid], ds_s[i * kC + tid], cfbar, xbar, abar);
            xs_s[i * kC + tid] = xbar;
            ds_s[i * kC + tid] = abar;
        }
    }

    // ---------------------------------------------------------------- reverse
    for (int q = 0; q < 9; ++q) cb_s[q * kC + tid] = 0.0;
    float gv[NT], inj[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) gv[t] = inj[t] = 0.f;
    float M0 = 0.f, M1 = 0.f, M2 = 0.f, I0 = 0.f, I1 = 0.f, I2 = 0.f;
    const float dtau = (float)(1.0 / P.m);
    const float a0 = Q.a0e, a1 = Q.a1e, a2 = Q.a2e, ce = Q.ce;
    float r0, r1, r2;  // normals drawn one step ahead (descending)
    draw_phi<float, false>(nullptr, gpath, active ? lp : 0, P.n_paths, n_steps - 1, P.rk0, P.rk1, r0, r1, r2);
    for (int i = B; i >= 2; --i) {
        {
            const float xb = xs_s[i * kC + tid], ab = ds_s[i * kC + tid];
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                if (t == i) {
                    inj[t] = ab;
                    gv[t] += xb;
                }
            }
            const float ti = dtau * (float)i;
            I0 += ab;
            I1 = fmaf(ab, ti, I1);
            I2 = fmaf(ab, ti * ti, I2);
            M0 += xb;
            M1 = fmaf(xb, ti, M1);
            M2 = fmaf(xb, ti * ti, M2);
        }
        float cbb[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) cbb[q] = 0.f;
        for (int n = i * stride - 1; n >= (i - 1) * stride; --n) {
            M0 += I0;
            M1 += I1;
            M2 += I2;
            const float phi0 = r0, phi1 = r1, phi2 = r2;
            draw_phi<float, false>(nullptr, gpath, active ? lp : 0, P.n_paths, max(n - 1, stride), P.rk0, P.rk1, r0,
                                   r1, r2);
            // v = g + inj: the adjoint of the state after step n; then g <- A2^T v,
            // descending in place (v[t-1], v[t-2] still unchanged)
#pragma unroll
            for (int t = 0; t < NT; ++t) gv[t] += inj[t];
            const float vL = gv[L], vL1 = gv[L - 1];
            if constexpr (POLY) {
                const float M2g = fmaf(Q.gL, vL, M2);
                cbb[0] = fmaf(phi0, M0, cbb[0]);
                cbb[1] = fmaf(phi0, M1, cbb[1]);
                cbb[2] = fmaf(phi0, M2g, cbb[2]);
                cbb[3] = fmaf(phi1, M0, cbb[3]);
                cbb[4] = fmaf(phi1, M1, cbb[4]);
                cbb[5] = fmaf(phi1, M2g, cbb[5]);
                cbb[6] = fmaf(phi2, M0, cbb[6]);
                cbb[7] = fmaf(phi2, M1, cbb[7]);
                cbb[8] = fmaf(phi2, M2g, cbb[8]);
            }
            gv[L] = fmaf(a2, gv[L - 2], fmaf(ce, vL1, (1.f + ce) * vL));
            gv[L - 1] = fmaf(a1, gv[L - 2], fmaf(a2, gv[L - 3], fmaf(1.f - ce, vL1, -ce * vL)));
#pragma unroll
            for (int t = L - 2; t >= 0; --t) {
                float y = a0 * gv[t];
                if (t >= 1) y = fmaf(a1, gv[t - 1], y);
                if (t >= 2) y = fmaf(a2, gv[t - 2], y);
                gv[t] = y;
            }
            M2 = fmaf(Q.wL, vL, fmaf(Q.wL1, vL1, fmaf(Q.k2p, M0, fmaf(Q.k1x2, M1, M2))));
            M1 = fmaf(Q.k1, M0, M1);
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) cb_s[q * kC + tid] += (double)cbb[q];
    }

    // ---------------------------------------------------------------- CTA reduction
    const int cx = B + 3, ca = 2 * B + 3, cc = 3 * B + 3;
    double* wred = red_s;
    __syncthreads();
    for (int i = 1; i <= B; ++i) {
        const double sx_ = warp_sum(active ? (double)xs_s[i * kC + tid] : 0.0);
        const double sa_ = warp_sum(active ? (double)ds_s[i * kC + tid] : 0.0);
        if (lane == 0) {
            wred[warp * R + cx + i - 1] = sx_;
            wred[warp * R + ca + i - 1] = sa_;
        }
    }
    for (int q = 0; q < 9; ++q) {
        const double sum = warp_sum(active ? cb_s[q * kC + tid] : 0.0);
        if (lane == 0) wred[warp * R + cc + q] = sum;
    }
    __syncthreads();
    for (int col = cx + tid; col < R; col += kC) {
        double sum = 0.0;
        for (int w = 0; w < kC / 32; ++w) sum += wred[w * R + col];
        partials[(size_t)blockIdx.x * R + col] = sum;
    }
}

size_t adjoint_pc_smem(int nt, int n_blocks) { return pc_adj_layout(nt, n_blocks, 3 * n_blocks + 12).total; }

template <int NT, bool POLY>
static cudaError_t launch_adj_pc_t(const PcParams<float>& Q, double* partials, cudaStream_t s)
{
    const size_t smem = adjoint_pc_smem(NT, Q.P.n_blocks);
    auto k = adjoint_kernel_pc<NT, POLY>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (Q.P.n_paths + kPcCta - 1) / kPcCta;
    k<<<(unsigned)grid, kPcCta, smem, s>>>(Q, partials);
    return cudaGetLastError();
}

cudaError_t launch_adjoint_pc(int nt, const PcParams<float>& Q, bool poly, double* partials, cudaStream_t s)
{
    if (nt == 51) return poly ? launch_adj_pc_t<51, true>(Q, partials, s) : launch_adj_pc_t<51, false>(Q, partials, s);
    if (nt == 61) return poly ? launch_adj_pc_t<61, true>(Q, partials, s) : launch_adj_pc_t<61, false>(Q, partials, s);
    return cudaErrorInvalidValue;
}

// ---------------------------------------------------------------------------
// The adjoint in the response form (Euler step, quadratic factors, the sampled
// states kept: checkpoint_every = 0).  The forward pass is the mixed
// valuation's response form (path_kernel_mixed_resp, hjm_mresp.cu: the parts
// S, U, W as FP32 scalars, the remainder as FP32 impulse-response sums in NS
// date slots, the same operations in the same order, so the path's cash
// flows are the valuation's); it keeps each date's sampled forward and
// discount factor.  The reverse sweep needs the per-tenor adjoint only for its
// last tenor, the remainder's coupling to W in the moment recursion
// (adjoint_kernel above): the adjoint of hc after step n at the last tenor is
//     g_n[L] = sum_j xbar_j G_j(n_j - n) + abar_j CG_j(n_j - n),
// G_j(m) = (A^m e_L)[j], CG_j its running sum, over the dates j still ahead
// of step n -- the forward table's own entries, so with the slot dates' seeds
// {xbar_j, abar_j} in registers the sweep's kappa g_n[L] is one packed FMA
// per slot (table row n) instead of the transposed convection of every tenor.
// Dates whose responses never count (no slot) contribute below 2^-30 of
// kappa per seed, as in the valuation.
// Shared memory: the cash flows (then the exposures, one row up) share their
// region with the sweep's coefficient sums, which start after the seeds have
// read the exposures (17.1 KB per CTA at 20 dates: 12 CTAs per SM, as the
// registers allow, instead of 10 with separate regions).
struct AdjRespLayout {
    size_t cf, cb, xs, ds, red, total;
};

__host__ __device__ inline AdjRespLayout adj_resp_layout(int B, int R)
{
    AdjRespLayout L;
    const size_t rows = (size_t)B + 1;
    const size_t cf = (rows + 1) * kAdjCta * 4, cb = (size_t)9 * kAdjCta * 8;
    L.cf = L.cb = 0;
    L.xs = align128(cf > cb ? cf : cb);
    L.ds = align128(L.xs + rows * kAdjCta * 4);
    L.red = align128(L.ds + rows * kAdjCta * 4);
    L.total = align128(L.red + (size_t)(kAdjCta / 32) * R * 8);
    return L;
}

// CTAs per SM the launch bounds ask for (8 slots: at 11 the compiler keeps
// 80 registers without spills, so 12 CTAs are resident, as the shared
// memory allows; asked for 12 it spills; 16 slots in 128 registers, 8)
constexpr int adj_resp_min_ctas(int ns) { return ns <= 8 ? 11 : 8; }

template <int NS>
__global__ void __launch_bounds__(kAdjCta, adj_resp_min_ctas(NS))
    adjoint_kernel_resp(const __grid_constant__ MixedParams M, const float4* __restrict__ resp,
                        double* __restrict__ partials)
{
    constexpr int C = kAdjCta;
    const PathParams<float>& P = M.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const int R = 3 * B + 12;
    const AdjRespLayout Ly = adj_resp_layout(B, R);
    float* cf_s = reinterpret_cast<float*>(smem + Ly.cf);  // [B+2][C]: cash flows, then exposures one row up
    float* xs_s = reinterpret_cast<float*>(smem + Ly.xs);  // [B+1][C]: x_i, then xbar_i
    float* ds_s = reinterpret_cast<float*>(smem + Ly.ds);  // [B+1][C]: D_i, then abar_i
    double* cb_s = reinterpret_cast<double*>(smem + Ly.cb);  // [9][C], the sweep's (over cf_s)
    double* red_s = reinterpret_cast<double*>(smem + Ly.red);

    const int64_t lp = (int64_t)blockIdx.x * C + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;
    const int stride = P.stride;
    const int n_steps = B * stride;

    // ---------------------------------------------------------------- forward
    float2 A[NS];  // {hc at date j's tenor, its running sum}, slot B - j
#pragma unroll
    for (int r = 0; r < NS; ++r) A[r] = make_float2(0.f, 0.f);
    float S = 0.f, U = 0.f, W = 0.f;
    double zS = 0.0, zU = 0.0, zW = 0.0;
    auto price = [&](int i, float2 rc) {
        const float ti = P.tau[i];
        const float pv = fmaf(ti, fmaf(ti, W, U), S);
        const double xv = P.psamp[i] + (double)(rc.x + pv);
        const double td = (double)ti;
        const double a = P.psum[i] + (double)rc.y + fma(td, fma(td, zW, zU), zS);
        const float D = expf((float)(-a * P.dt));
        const float mm = (float)P.m;
        const float L = mm * expm1f((float)xv / mm);
        cf_s[i * C + tid] = D * ((float)P.payA[i] * L - (float)P.payB[i]);
        xs_s[i * C + tid] = (float)xv;
        ds_s[i * C + tid] = D;
    };
    price(1, make_float2(0.f, 0.f));
    const int n_last = n_steps - 1;
    float q0, q1, q2;
    draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, min(stride, n_last), P.rk0, P.rk1, q0, q1, q2);
    for (int b = 1; b < B; ++b) {
        float sS = 0.f, sU = 0.f, sW = 0.f;
        const float4* row = resp + (size_t)b * stride * (NS / 2);
#pragma unroll 5  // (a divisor of 50 steps per block: 8.66 ms against 8.77 by 2 at 1M paths)
        for (int s = 0; s < stride; ++s) {
            const int n = b * stride + s;
            const float phi0 = q0, phi1 = q1, phi2 = q2;
            draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, min(n + 1, n_last), P.rk0, P.rk1, q0, q1, q2);
            const float2 w2 = make_float2(W, W);
            const float4* rr = row + (size_t)s * (NS / 2);
#pragma unroll
            for (int u = 0; u < NS / 2; ++u) {
                const float4 e = __ldg(rr + u);
                A[2 * u] = __ffma2_rn(make_float2(e.x, e.y), w2, A[2 * u]);
                A[2 * u + 1] = __ffma2_rn(make_float2(e.z, e.w), w2, A[2 * u + 1]);
            }
            float Sn = fmaf(M.svcf[0][0], phi0, fmaf(M.k2f, W, fmaf(M.k1f, U, S)));
            Sn = fmaf(M.svcf[2][0], phi2, fmaf(M.svcf[1][0], phi1, Sn));
            float Un = fmaf(M.svcf[1][1], phi1, fmaf(M.svcf[0][1], phi0, fmaf(2.0f * M.k1f, W, U)));
            Un = fmaf(M.svcf[2][1], phi2, Un);
            const float Wn = fmaf(M.svcf[2][2], phi2, fmaf(M.svcf[1][2], phi1, fmaf(M.svcf[0][2], phi0, W)));
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
        const int r = B - (b + 1);
        price(b + 1, r < NS ? select_reg<NS, float2>(A, r) : make_float2(0.f, 0.f));
    }

    // exposures, the path's CVA contribution, the CTA's EE and CVA partial sums
    float* e_s = cf_s + C;
    double v = 0.0, cva_c = 0.0;
    e_s[B * C + tid] = 0.f;
    for (int j = B - 1; j >= 0; --j) {
        v += (double)cf_s[(j + 1) * C + tid];
        double e = (v > 0.0) ? v : 0.0;
        if (!active) e = 0.0;
        e_s[j * C + tid] = (float)e;
        cva_c = fma(P.cvaw[j], e, cva_c);
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    for (int j = warp; j <= B; j += C / 32) {
        double sum = 0.0;
#pragma unroll
        for (int q = 0; q < C / 32; ++q) sum += (double)e_s[j * C + lane + 32 * q];
        sum = warp_sum(sum);
        if (lane == 0) partials[(size_t)blockIdx.x * R + j] = sum;
    }
    {
        const double s1 = warp_sum(cva_c), s2 = warp_sum(cva_c * cva_c);
        if (lane == 0) {
            red_s[warp] = s1;
            red_s[C / 32 + warp] = s2;
        }
    }
    __syncthreads();
    if (tid == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < C / 32; ++w) {
            s1 += red_s[w];
            s2 += red_s[C / 32 + w];
        }
        partials[(size_t)blockIdx.x * R + B + 1] = s1;
        partials[(size_t)blockIdx.x * R + B + 2] = s2;
    }
    __syncthreads();  // (red_s is reused by the final reduction)

    // per-date seeds from cfbar_i = sum_{j<i} w_j [E_j > 0]
    {
        float cfbar = 0.f;
        for (int i = 1; i <= B; ++i) {
            const int j = i - 1;
            if (e_s[j * C + tid] > 0.f) cfbar += (float)P.cvaw[j];
            if (!active) cfbar = 0.f;
            float xbar, abar;
            date_seeds(P, i, (double)xs_s[i * C + tid], ds_s[i * C + tid], cfbar, xbar, abar);
            xs_s[i * C + tid] = xbar;
            ds_s[i * C + tid] = abar;
        }
    }

    // ---------------------------------------------------------------- reverse
    __syncthreads();  // (cb_s overlays the exposures that the seeds just read)
    for (int q = 0; q < 9; ++q) cb_s[q * C + tid] = 0.0;
    float2 sd[NS];  // {xbar_j, abar_j} of slot r's date j = B - r once the sweep reaches it
#pragma unroll
    for (int r = 0; r < NS; ++r) sd[r] = make_float2(0.f, 0.f);
    float M0 = 0.f, M1 = 0.f, M2 = 0.f, I0 = 0.f, I1 = 0.f, I2 = 0.f;
    const float dtau = (float)(1.0 / P.m);
    const float k1 = P.c * dtau, k2 = P.c * dtau * dtau;
    float r0, r1, r2;
    draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, n_steps - 1, P.rk0, P.rk1, r0, r1, r2);
    for (int i = B; i >= 2; --i) {
        {
            const float xb = xs_s[i * C + tid], ab = ds_s[i * C + tid];
            const int rs = B - i;
#pragma unroll
            for (int r = 0; r < NS; ++r)
                if (r == rs) sd[r] = make_float2(xb, ab);
            const float ti = dtau * (float)i;
            I0 += ab;
            I1 = fmaf(ab, ti, I1);
            I2 = fmaf(ab, ti * ti, I2);
            M0 += xb;
            M1 = fmaf(xb, ti, M1);
            M2 = fmaf(xb, ti * ti, M2);
        }
        float cbb[9];
#pragma unroll
        for (int q = 0; q < 9; ++q) cbb[q] = 0.f;
#pragma unroll 2
        for (int n = i * stride - 1; n >= (i - 1) * stride; --n) {
            M0 += I0;
            M1 += I1;
            M2 += I2;
            const float phi0 = r0, phi1 = r1, phi2 = r2;
            draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, max(n - 1, stride), P.rk0, P.rk1, r0, r1, r2);
            cbb[0] = fmaf(phi0, M0, cbb[0]);
            cbb[1] = fmaf(phi0, M1, cbb[1]);
            cbb[2] = fmaf(phi0, M2, cbb[2]);
            cbb[3] = fmaf(phi1, M0, cbb[3]);
            cbb[4] = fmaf(phi1, M1, cbb[4]);
            cbb[5] = fmaf(phi1, M2, cbb[5]);
            cbb[6] = fmaf(phi2, M0, cbb[6]);
            cbb[7] = fmaf(phi2, M1, cbb[7]);
            cbb[8] = fmaf(phi2, M2, cbb[8]);
            // kappa g_n[L] from the slot dates' seeds and table row n
            float2 kg = make_float2(0.f, 0.f);
            const float4* rr = resp + (size_t)n * (NS / 2);
#pragma unroll
            for (int u = 0; u < NS / 2; ++u) {
                const float4 e = __ldg(rr + u);
                kg = __ffma2_rn(make_float2(e.x, e.y), sd[2 * u], kg);
                kg = __ffma2_rn(make_float2(e.z, e.w), sd[2 * u + 1], kg);
            }
            M2 = fmaf(k2, M0, fmaf(2.f * k1, M1, M2)) + (kg.x + kg.y);
            M1 = fmaf(k1, M0, M1);
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) cb_s[q * C + tid] += (double)cbb[q];
    }

    // ---------------------------------------------------------------- CTA reduction
    // columns as adjoint_kernel's: [0..B] EE, B+1/B+2 CVA stats, E xbar_i,
    // E abar_i (i = 1..B), the 9 coefficient columns
    const int cx = B + 3, ca = 2 * B + 3, cc = 3 * B + 3;
    double* wred = red_s;  // [warp][R]
    for (int i = 1; i <= B; ++i) {
        const double sx_ = warp_sum(active ? (double)xs_s[i * C + tid] : 0.0);
        const double sa_ = warp_sum(active ? (double)ds_s[i * C + tid] : 0.0);
        if (lane == 0) {
            wred[warp * R + cx + i - 1] = sx_;
            wred[warp * R + ca + i - 1] = sa_;
        }
    }
    for (int q = 0; q < 9; ++q) {
        const double sum = warp_sum(active ? cb_s[q * C + tid] : 0.0);
        if (lane == 0) wred[warp * R + cc + q] = sum;
    }
    __syncthreads();
    for (int col = cx + tid; col < R; col += C) {
        double sum = 0.0;
        for (int w = 0; w < C / 32; ++w) sum += wred[w * R + col];
        partials[(size_t)blockIdx.x * R + col] = sum;
    }
}

size_t adjoint_resp_smem(int n_blocks) { return adj_resp_layout(n_blocks, 3 * n_blocks + 12).total; }

cudaError_t launch_adjoint_resp(const AdjParams& A, int ns, const float4* table, double* partials, cudaStream_t s)
{
    if (ns != 8 && ns != 16) return cudaErrorInvalidValue;
    const int B = A.M.P.n_blocks;
    if (B < 1 || B >= kMaxTenor || A.M.P.stride < 1) return cudaErrorInvalidValue;
    auto k = ns == 8 ? adjoint_kernel_resp<8> : adjoint_kernel_resp<16>;
    const size_t smem = adjoint_resp_smem(B);
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (A.M.P.n_paths + kAdjCta - 1) / kAdjCta;
    k<<<(unsigned)grid, kAdjCta, smem, s>>>(A.M, table, partials);
    return cudaGetLastError();
}

size_t adjoint_smem(int nt, int n_blocks, bool ckpt) { return adj_layout(nt, n_blocks, 3 * n_blocks + 12, ckpt).total; }

int adjoint_columns(int nt, int n_blocks)
{
    (void)nt;
    return 3 * n_blocks + 12;
}

int adjoint_cta() { return kAdjCta; }

template <int NT, bool CKPT, bool POLY>
static cudaError_t launch_adj_t(const AdjParams& A, double* partials, float* ck_h, double* ck_a, cudaStream_t s)
{
    const size_t smem = adjoint_smem(NT, A.M.P.n_blocks, CKPT);
    auto k = adjoint_kernel<NT, CKPT, POLY>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (A.M.P.n_paths + kAdjCta - 1) / kAdjCta;
    k<<<(unsigned)grid, kAdjCta, smem, s>>>(A, partials, ck_h, ck_a);
    return cudaGetLastError();
}

template <int NT>
static cudaError_t launch_adj_nt(const AdjParams& A, bool poly, double* partials, float* ck_h, double* ck_a,
                                 cudaStream_t s)
{
    const bool ck = A.ckpt_every > 0;
    if (poly) return ck ? launch_adj_t<NT, true, true>(A, partials, ck_h, ck_a, s)
                        : launch_adj_t<NT, false, true>(A, partials, ck_h, ck_a, s);
    return ck ? launch_adj_t<NT, true, false>(A, partials, ck_h, ck_a, s)
              : launch_adj_t<NT, false, false>(A, partials, ck_h, ck_a, s);
}

cudaError_t launch_adjoint(int nt, const AdjParams& A, bool poly, double* partials, float* ck_h, double* ck_a,
                           cudaStream_t s)
{
    if (nt == 51) return launch_adj_nt<51>(A, poly, partials, ck_h, ck_a, s);
    if (nt == 61) return launch_adj_nt<61>(A, poly, partials, ck_h, ck_a, s);
    return cudaErrorInvalidValue;
}

}  // namespace hjm
