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
// The Jacobian A does not depend on the state, so the same g serves p and h,
// and the sweep needs no forward state beyond the per-date seeds:
//     dCVA/dspot      = g_{stride-1} + (stride-1) abar          (block 0 holds spot)
//     dCVA/dmu[t]     = dt sum_{n >= stride} g_n[t]
//     dCVA/dS[t][k]   = sum_n g_n[t] phi_{n,k}
// and with sigma_k(T) = sum_d c_{k,d} T^d the volatility coefficients need only
// the three moments M_d(n) = sum_t g_n[t] tau_t^d per step:
//     dCVA/dc_{k,d} (diffusion) = sqrt(dt) sum_n phi_{n,k} M_d(n).
// The drift's own dependence on the coefficients (trapezoid rule) is chained
// on the host.  The normals are regenerated from their Philox counters.
//
// Checkpoint mode (checkpoint_every = K in [1, stride]).  The forward pass
// keeps only the cash flows; it writes the stochastic curve h and the FP64
// discount sum of the next tenor to be sampled to HBM before every K-th
// Euler step.  The reverse sweep walks the segments backwards, reloads the
// segment's checkpoint, recomputes the segment's states forward (regenerated
// normals) to rebuild the sampled forward and discount of the date that falls
// inside it, and then sweeps the segment backwards.  With K = 0 the forward
// pass keeps the per-date (x_i, D_i) instead and nothing is recomputed.
#include <cuda_runtime.h>

#include <cstdint>

#include "hjm_device.cuh"
#include "hjm_kernels.h"

namespace hjm {

// Shared memory per CTA (thread-private columns):
//   region A  [cf_s (B+1) f32 | acc_s (B+1) f64 | work_s (max(NT,B+1)) f32],
//             overlaid by mu_s (NT f64) during the reverse sweep
//   xs_s      (B+1) f32    K = 0: x_i then xbar_i;  K > 0: cfbar_i
//   ds_s      (B+1) f32    K = 0: D_i then abar_i
//   cb_s      9 f64        diffusion coefficient adjoints
//   red_s     (kCta/32) * R f64   CTA reduction
struct AdjLayout {
    size_t cf, acc, work, mu, xs, ds, cb, red, total;
};

__host__ __device__ inline size_t align128(size_t x) { return (x + 127) & ~(size_t)127; }

__host__ __device__ inline AdjLayout adj_layout(int nt, int B, int R)
{
    AdjLayout L;
    const size_t rows = (size_t)B + 1, wrows = (size_t)(nt > B + 1 ? nt : B + 1);
    L.cf = 0;
    L.acc = align128(rows * kCta * 4);
    L.work = align128(L.acc + rows * kCta * 8);
    size_t endA = L.work + wrows * kCta * 4;
    const size_t mu_bytes = (size_t)nt * kCta * 8;
    if (endA < mu_bytes) endA = mu_bytes;
    L.mu = 0;
    L.xs = align128(endA);
    L.ds = align128(L.xs + rows * kCta * 4);
    L.cb = align128(L.ds + rows * kCta * 4);
    L.red = align128(L.cb + (size_t)9 * kCta * 8);
    L.total = align128(L.red + (size_t)(kCta / 32) * R * 8);
    return L;
}

// g <- A^T g for the upwind convection operator A of euler_step:
//   (A h)[t] = h[t] + c (h[t+1] - h[t]) (t < L),  (A h)[L] = h[L] + c (h[L] - h[L-1]).
template <int NT>
__device__ __forceinline__ void adjoint_convection(float (&g)[NT], float c)
{
    constexpr int L = NT - 1;
    float gn[NT];
    gn[0] = fmaf(-c, g[0], g[0]);
#pragma unroll
    for (int t = 1; t <= L - 2; ++t) gn[t] = fmaf(c, g[t - 1] - g[t], g[t]);
    gn[L - 1] = fmaf(-c, g[L], fmaf(c, g[L - 2] - g[L - 1], g[L - 1]));
    gn[L] = fmaf(c, g[L] + g[L - 1], g[L]);
#pragma unroll
    for (int t = 0; t < NT; ++t) g[t] = gn[t];
}

// Seeds of date i from its sampled forward x, discount factor D and cfbar.
__device__ __forceinline__ void date_seeds(const AdjParams& A, int i, double x, float D, float cfbar, float& xbar,
                                           float& abar)
{
    const float mm = (float)A.P.m;
    const float xf = (float)x;
    const float e = expf(xf / mm);
    const float L = mm * expm1f(xf / mm);
    const float pa = (float)A.P.payA[i], pbk = (float)A.P.payB[i];
    xbar = cfbar * D * pa * e;
    abar = -(float)A.P.dt * D * cfbar * (pa * L - pbk);
}

template <int NT, bool CKPT>
__global__ void __launch_bounds__(kCta, 2)
    adjoint_kernel(const __grid_constant__ AdjParams A, double* __restrict__ partials, float* __restrict__ ck_h,
                   double* __restrict__ ck_a)
{
    const PathParams<float>& P = A.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const int rows = B + 1;
    const int R = B + 3 + 2 * NT + 9;
    const AdjLayout Ly = adj_layout(NT, B, R);
    float* cf_s = reinterpret_cast<float*>(smem + Ly.cf);
    double* acc_s = reinterpret_cast<double*>(smem + Ly.acc);
    float* work_s = reinterpret_cast<float*>(smem + Ly.work);
    double* mu_s = reinterpret_cast<double*>(smem + Ly.mu);
    float* xs_s = reinterpret_cast<float*>(smem + Ly.xs);
    float* ds_s = reinterpret_cast<float*>(smem + Ly.ds);
    double* cb_s = reinterpret_cast<double*>(smem + Ly.cb);
    double* red_s = reinterpret_cast<double*>(smem + Ly.red);

    const int64_t lp = (int64_t)blockIdx.x * kCta + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;
    const int stride = P.stride;
    const int n_steps = B * stride;
    const int K = CKPT ? A.ckpt_every : stride;
    const float c = P.c;
    const int64_t ld = A.ck_ld;

    // ------------------------------------------------------------ forward
    float h[NT], pb[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        h[t] = 0.f;
        pb[t] = 0.f;
    }
    for (int i = 0; i < rows; ++i) acc_s[i * kCta + tid] = 0.0;

    auto sample_fwd = [&](int i) {
        const float hi = select_reg<NT, float>(h, i);
        const double x = P.psamp[i] + (double)hi;
        const double a = P.psum[i] + acc_s[i * kCta + tid];
        const float D = expf((float)(-a * P.dt));
        const float mm = (float)P.m;
        const float L = mm * expm1f((float)x / mm);
        cf_s[i * kCta + tid] = D * ((float)P.payA[i] * L - (float)P.payB[i]);
        if (!CKPT) {
            xs_s[i * kCta + tid] = (float)x;
            ds_s[i * kCta + tid] = D;
        }
    };

    sample_fwd(1);
    for (int b = 1; b < B; ++b) {
        for (int s = 0; s < stride; ++s) {
            const int n = b * stride + s;
            if (CKPT && ((n - stride) % K) == 0) {
                // checkpoint before step n: the curve and the discount sum of the
                // next tenor to be sampled (completed blocks + current partial)
                const int ck = (n - stride) / K;
                const int inext = (n + stride) / stride;
                if (active) {
#pragma unroll
                    for (int t = 0; t < NT; ++t) ck_h[((size_t)ck * NT + t) * ld + lp] = h[t];
                    ck_a[(size_t)ck * ld + lp] =
                        acc_s[inext * kCta + tid] + (double)select_reg<NT, float>(pb, inext);
                }
            }
            float phi0, phi1, phi2;
            draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, n, P.rk0, P.rk1, phi0, phi1, phi2);
            euler_step<NT, float>(h, P, c, phi0, phi1, phi2);
#pragma unroll
            for (int t = 1; t < NT; ++t) pb[t] += h[t];
        }
#pragma unroll
        for (int t = 1; t < NT; ++t) {
            work_s[t * kCta + tid] = pb[t];
            pb[t] = 0.f;
        }
        for (int t = b + 1; t <= B; ++t) acc_s[t * kCta + tid] += (double)work_s[t * kCta + tid];
        sample_fwd(b + 1);
    }

    // exposures, CVA contribution, cash-flow adjoints
    float* e_s = work_s;
    double v = 0.0, cva_c = 0.0;
    e_s[B * kCta + tid] = 0.f;
    for (int j = B - 1; j >= 0; --j) {
        v += (double)cf_s[(j + 1) * kCta + tid];
        double e = (v > 0.0) ? v : 0.0;
        if (!active) e = 0.0;
        e_s[j * kCta + tid] = (float)e;
        cva_c = fma(P.cvaw[j], e, cva_c);
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    for (int j = warp; j <= B; j += kCta / 32) {
        double s = 0.0;
#pragma unroll
        for (int q = 0; q < kCta / 32; ++q) s += (double)e_s[j * kCta + lane + 32 * q];
        s = warp_sum(s);
        if (lane == 0) partials[(size_t)blockIdx.x * R + j] = s;
    }
    {
        const double s1 = warp_sum(cva_c), s2 = warp_sum(cva_c * cva_c);
        if (lane == 0) {
            red_s[warp] = s1;
            red_s[kCta / 32 + warp] = s2;
        }
    }
    __syncthreads();
    if (tid == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kCta / 32; ++w) {
            s1 += red_s[w];
            s2 += red_s[kCta / 32 + w];
        }
        partials[(size_t)blockIdx.x * R + B + 1] = s1;
        partials[(size_t)blockIdx.x * R + B + 2] = s2;
    }

    // cfbar_i = sum_{j<i} w_j [E_j > 0]; per-date seeds (K = 0) or cfbar kept (K > 0)
    {
        float cfbar = 0.f;
        for (int i = 1; i <= B; ++i) {
            const int j = i - 1;
            if (e_s[j * kCta + tid] > 0.f) cfbar += (float)P.cvaw[j];
            if (!active) cfbar = 0.f;
            if (CKPT) {
                xs_s[i * kCta + tid] = cfbar;
            } else {
                float xbar, abar;
                date_seeds(A, i, (double)xs_s[i * kCta + tid], ds_s[i * kCta + tid], cfbar, xbar, abar);
                xs_s[i * kCta + tid] = xbar;
                ds_s[i * kCta + tid] = abar;
            }
        }
    }
    __syncthreads();  // region A becomes mu_s

    // ------------------------------------------------------------ reverse
    for (int t = 0; t < NT; ++t) mu_s[t * kCta + tid] = 0.0;
    for (int q = 0; q < 9; ++q) cb_s[q * kCta + tid] = 0.0;
    float g[NT], inj[NT], mub[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        g[t] = 0.f;
        inj[t] = 0.f;
        mub[t] = 0.f;
    }
    float cbb[9];
#pragma unroll
    for (int q = 0; q < 9; ++q) cbb[q] = 0.f;

    const int E = n_steps - stride;                 // evolving steps
    const int S = (E + K - 1) / K;                  // segments
    for (int sg = S - 1; sg >= 0; --sg) {
        const int n0 = stride + sg * K;
        const int n1 = (n0 + K < n_steps) ? n0 + K : n_steps;
        int idate = 0;
        float sx = 0.f, sa = 0.f;
        if (CKPT) {
            // recompute the segment from its checkpoint; rebuild the seeds of
            // the date sampled inside it (at most one, since K <= stride)
            float hr[NT], pbr[NT];
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                hr[t] = active ? ck_h[((size_t)sg * NT + t) * ld + lp] : 0.f;
                pbr[t] = 0.f;
            }
            const int inext = (n0 + stride) / stride;
            const double a0 = active ? ck_a[(size_t)sg * ld + lp] : 0.0;
            for (int n = n0; n < n1; ++n) {
                float phi0, phi1, phi2;
                draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, n, P.rk0, P.rk1, phi0, phi1, phi2);
                euler_step<NT, float>(hr, P, c, phi0, phi1, phi2);
#pragma unroll
                for (int t = 1; t < NT; ++t) pbr[t] += hr[t];
                if ((n + 1) % stride == 0) {
                    const int i = (n + 1) / stride;  // == inext
                    const double x = P.psamp[i] + (double)select_reg<NT, float>(hr, i);
                    const double a = P.psum[i] + a0 + (double)select_reg<NT, float>(pbr, i);
                    const float D = expf((float)(-a * P.dt));
                    date_seeds(A, i, x, D, xs_s[i * kCta + tid], sx, sa);
                    idate = i;
                }
            }
            (void)inext;
        }
        for (int n = n1 - 1; n >= n0; --n) {
            // seeds of step n: a sampling step turns on tenor i's discount seed
            if ((n + 1) % stride == 0) {
                const int i = (n + 1) / stride;
                float xb, ab;
                if (CKPT) {
                    xb = (i == idate) ? sx : 0.f;
                    ab = (i == idate) ? sa : 0.f;
                } else {
                    xb = xs_s[i * kCta + tid];
                    ab = ds_s[i * kCta + tid];
                }
#pragma unroll
                for (int t = 1; t < NT; ++t) {
                    if (t == i) {
                        inj[t] = ab;
                        g[t] += xb;
                    }
                }
            }
#pragma unroll
            for (int t = 0; t < NT; ++t) g[t] += inj[t];
            // accumulate: drift adjoint and the three basis moments of g
            float m0a = 0.f, m0b = 0.f, m1a = 0.f, m1b = 0.f, m2a = 0.f, m2b = 0.f;
#pragma unroll
            for (int t = 0; t < NT; ++t) {
                mub[t] += g[t];
                if (t & 1) {
                    m0b += g[t];
                    m1b = fmaf(g[t], A.tau[t], m1b);
                    m2b = fmaf(g[t], A.tau2[t], m2b);
                } else {
                    m0a += g[t];
                    m1a = fmaf(g[t], A.tau[t], m1a);
                    m2a = fmaf(g[t], A.tau2[t], m2a);
                }
            }
            const float m0 = m0a + m0b, m1 = m1a + m1b, m2 = m2a + m2b;
            float phi0, phi1, phi2;
            draw_phi<float, false>(nullptr, gpath, lp, P.n_paths, n, P.rk0, P.rk1, phi0, phi1, phi2);
            cbb[0] = fmaf(phi0, m0, cbb[0]);
            cbb[1] = fmaf(phi0, m1, cbb[1]);
            cbb[2] = fmaf(phi0, m2, cbb[2]);
            cbb[3] = fmaf(phi1, m0, cbb[3]);
            cbb[4] = fmaf(phi1, m1, cbb[4]);
            cbb[5] = fmaf(phi1, m2, cbb[5]);
            cbb[6] = fmaf(phi2, m0, cbb[6]);
            cbb[7] = fmaf(phi2, m1, cbb[7]);
            cbb[8] = fmaf(phi2, m2, cbb[8]);
            adjoint_convection<NT>(g, c);
        }
        // fold the segment's FP32 partials into the FP64 accumulators
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            mu_s[t * kCta + tid] += (double)mub[t];
            mub[t] = 0.f;
        }
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            cb_s[q * kCta + tid] += (double)cbb[q];
            cbb[q] = 0.f;
        }
    }
    // seeds of step stride-1 (date 1 is deterministic: h = 0 through block 0)
    {
        const double x1 = P.psamp[1];
        const float D1 = expf((float)(-P.psum[1] * P.dt));
        float xb, ab;
        const float cfbar1 = CKPT ? xs_s[1 * kCta + tid] : 0.f;
        if (CKPT) {
            date_seeds(A, 1, x1, D1, cfbar1, xb, ab);
        } else {
            xb = xs_s[1 * kCta + tid];
            ab = ds_s[1 * kCta + tid];
        }
        inj[1] = ab;
        g[1] += xb;
    }
    // dCVA/dspot = g_{stride-1} + (stride - 1) * abar  (steps 0 .. stride-2 read spot directly)
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        g[t] += inj[t];
        g[t] = fmaf((float)(stride - 1), inj[t], g[t]);
        if (!active) g[t] = 0.f;
    }

    // ------------------------------------------------------------ CTA reduction
    // columns: [0..B] EE, B+1/B+2 CVA stats (written above),
    // B+3 .. B+2+NT spot, then NT drift, then 9 coefficient columns
    const int cs = B + 3, cm = B + 3 + NT, cc = B + 3 + 2 * NT;
    double* wred = red_s;  // [warp][R]
#pragma unroll
    for (int t = 0; t < NT; ++t) {
        const double s = warp_sum((double)g[t]);
        if (lane == 0) wred[warp * R + cs + t] = s;
    }
    for (int t = 0; t < NT; ++t) {
        const double s = warp_sum(active ? mu_s[t * kCta + tid] : 0.0);
        if (lane == 0) wred[warp * R + cm + t] = s;
    }
    for (int q = 0; q < 9; ++q) {
        const double s = warp_sum(active ? cb_s[q * kCta + tid] : 0.0);
        if (lane == 0) wred[warp * R + cc + q] = s;
    }
    __syncthreads();
    for (int col = cs + tid; col < R; col += kCta) {
        double s = 0.0;
        for (int w = 0; w < kCta / 32; ++w) s += wred[w * R + col];
        partials[(size_t)blockIdx.x * R + col] = s;
    }
}

size_t adjoint_smem(int nt, int n_blocks)
{
    return adj_layout(nt, n_blocks, n_blocks + 3 + 2 * nt + 9).total;
}

int adjoint_columns(int nt, int n_blocks) { return n_blocks + 3 + 2 * nt + 9; }

template <int NT, bool CKPT>
static cudaError_t launch_adj_t(const AdjParams& A, double* partials, float* ck_h, double* ck_a, cudaStream_t s)
{
    const size_t smem = adjoint_smem(NT, A.P.n_blocks);
    auto k = adjoint_kernel<NT, CKPT>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (A.P.n_paths + kCta - 1) / kCta;
    k<<<(unsigned)grid, kCta, smem, s>>>(A, partials, ck_h, ck_a);
    return cudaGetLastError();
}

cudaError_t launch_adjoint(int nt, const AdjParams& A, double* partials, float* ck_h, double* ck_a, cudaStream_t s)
{
    const bool ck = A.ckpt_every > 0;
    if (nt == 51) return ck ? launch_adj_t<51, true>(A, partials, ck_h, ck_a, s)
                            : launch_adj_t<51, false>(A, partials, ck_h, ck_a, s);
    if (nt == 61) return ck ? launch_adj_t<61, true>(A, partials, ck_h, ck_a, s)
                            : launch_adj_t<61, false>(A, partials, ck_h, ck_a, s);
    return cudaErrorInvalidValue;
}

}  // namespace hjm
