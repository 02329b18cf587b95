// hjm_pc.cu -- the predictor-corrector (Heun) time scheme for the Musiela SDE.
//
// New work: the reference evolves the curve with the Euler step of
// simulation_cpu.h:37-54 and lists a predictor-corrector as a to-do
// (doc/TODO:3).  With deterministic volatilities the corrector acts on the
// drift term a(f) = mu + D f (D the forward difference / dtau, backward at the
// last tenor L):  f* = f + a(f) dt + xi,  f' = f + (a(f) + a(f*)) dt / 2 + xi,
// which is linear:  f' = A2 f + N (mu dt + xi),  A2 = I + c Dl + c^2 Dl^2 / 2,
// N = I + c Dl / 2 (Dl = dtau D, c = dt / dtau).  Per tenor t <= L-2,
//     (A2 h)[t] = a0 h[t] + a1 h[t+1] + a2 h[t+2],
//     a0 = 1 - c + c^2/2,  a1 = c - c^2,  a2 = c^2/2,
// and rows L-1, L are the Euler rows (Dl^2 vanishes there).  The curve split
// f = p + h keeps p (drift, FP64, host) out of the kernel; the noise enters
// through the loadings N sqrt(dt) sigma (host).
//
// Growth scaling as in the Euler kernels: with v = h base^n', the interior
// step is v + r1 v[t+1] + r2 v[t+2] (two FMAs per tenor), r1 = a1/a0 and
// r2 = a2/a0 rounded once, and base = 1 + r1 + r2; the effective scheme is
// a0 = 1/base, a1 = r1/base, a2 = r2/base, and the boundary rows are written
// in r1, r2 so that constant curves grow by exactly base everywhere:
//     v'[L-1] = v[L-1] + r1 v[L] + r2 (2 v[L] - v[L-1]),
//     v'[L]   = v[L] + r1 (2 v[L] - v[L-1]) + r2 (3 v[L] - 2 v[L-1]).
// Discount integrals: block sums recovered from (I - A2) H = X - A2 d (X the
// block's injected noise, d = h_end - h_start), downward from the directly
// accumulated last tenor: row L-1 is two-point, rows t <= L-2 average H[t+1]
// and H[t+2] with weights summing to one (stable).  One kernel for both
// precisions: T = double (FP64) or float (mixed: FP32 curve, pricing and
// block sums, FP64 discount accumulation and reductions).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "hjm_device.cuh"
#include "hjm_epilogue.cuh"
#include "hjm_kernels.h"
#include "hjm_pc.cuh"
#include "hjm_resp.cuh"

namespace hjm {

// Shared memory per thread (columns of kPcCta): acc (B+1) FP64, slot i the
// discount sum of tenor i until date i is sampled, then its cash flow; hs
// (NT) T, the curve at the block start, reused for the exposure tile.
__host__ __device__ inline size_t pc_smem_bytes(int nt, int n_blocks, size_t tsize)
{
    size_t b = ((size_t)n_blocks + 1) * kPcCta * 8;
    b = (b + 127) & ~(size_t)127;
    b += (size_t)(nt > n_blocks + 1 ? nt : n_blocks + 1) * kPcCta * tsize;
    b = (b + 127) & ~(size_t)127;
    return b + 2 * (kPcCta / 32) * 8;
}

template <int NT, typename T, bool EXT, bool POLY>
__global__ void __launch_bounds__(kPcCta, 4)
    path_kernel_pc(const __grid_constant__ PcParams<T> Q, const double* __restrict__ ext,
                   double* __restrict__ partials, T* __restrict__ estore)
{
    const PathParams<T>& P = Q.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    double* acc_s = reinterpret_cast<double*>(smem);
    const size_t off = (((size_t)B + 1) * kPcCta * 8 + 127) & ~(size_t)127;
    T* hs_s = reinterpret_cast<T*>(smem + off);
    const size_t hs_rows = (size_t)(NT > B + 1 ? NT : B + 1);
    double* red_s = reinterpret_cast<double*>(smem + ((off + hs_rows * kPcCta * sizeof(T) + 127) & ~(size_t)127));

    const int64_t cta_base = (int64_t)blockIdx.x * kPcCta;
    const int64_t lp = cta_base + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;

    PcPath<NT, T, POLY> x;
    x.reset();
    for (int i = 0; i <= B; ++i) acc_s[i * kPcCta + tid] = 0.0;
    for (int t = 0; t < NT; ++t) hs_s[t * kPcCta + tid] = T(0);

    auto sample = [&](int i) {
        const double xv = P.psamp[i] + (double)x.value(P, i);
        const double a = P.psum[i] + acc_s[i * kPcCta + tid];
        const T D = exp_t<T>((T)(-a * P.dt));
        const T mm = (T)P.m;
        const T Lb = mm * expm1_t<T>((T)xv / mm);
        acc_s[i * kPcCta + tid] = (double)(D * ((T)P.payA[i] * Lb - (T)P.payB[i]));
    };

    sample(1);
    for (int b = 1; b < B; ++b) {
        x.begin_block(P, b);
        for (int s = 0; s < P.stride; ++s) {
            const int n = b * P.stride + s;
            T phi0, phi1, phi2;
            draw_phi<T, EXT>(ext, gpath, active ? lp : 0, P.n_paths, n, P.rk0, P.rk1, phi0, phi1, phi2);
            x.step(Q, phi0, phi1, phi2);
        }
        x.end_block(Q, b, B, hs_s, acc_s, tid);
        sample(b + 1);
    }

    // exposures E_j = max(sum_{i>j} cf_i, 0) (FP64 suffix sums), the path's
    // CVA contribution, CTA partial sums, optional exposure rows to HBM
    T* e_s = hs_s;
    double vs = 0.0, cva_c = 0.0;
    e_s[B * kPcCta + tid] = T(0);
    for (int j = B - 1; j >= 0; --j) {
        vs += acc_s[(j + 1) * kPcCta + tid];
        double e = (vs > 0.0) ? vs : 0.0;
        if (!active) e = 0.0;
        e_s[j * kPcCta + tid] = (T)e;
        cva_c = fma(P.cvaw[j], e, cva_c);
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    const int R = B + 3;
    for (int j = warp; j <= B; j += kPcCta / 32) {
        double sum = 0.0;
#pragma unroll
        for (int q = 0; q < kPcCta / 32; ++q) sum += (double)e_s[j * kPcCta + lane + 32 * q];
        sum = warp_sum(sum);
        if (lane == 0) partials[(size_t)blockIdx.x * R + j] = sum;
    }
    {
        const double s1 = warp_sum(cva_c), s2 = warp_sum(cva_c * cva_c);
        if (lane == 0) {
            red_s[warp] = s1;
            red_s[kPcCta / 32 + warp] = s2;
        }
    }
    if (P.store_exposures) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kPcCta / 32; ++w) {
            s1 += red_s[w];
            s2 += red_s[kPcCta / 32 + w];
        }
        partials[(size_t)blockIdx.x * R + B + 1] = s1;
        partials[(size_t)blockIdx.x * R + B + 2] = s2;
        if (P.store_exposures) {
            // date rows of this CTA's paths, smem -> HBM with the bulk-copy (TMA) engine;
            // rows padded to 16 bytes (the store's row stride ld is a multiple of 4)
            constexpr int kPad = 16 / (int)sizeof(T);
            const int64_t cnt = (P.n_paths - cta_base < kPcCta) ? (P.n_paths - cta_base) : kPcCta;
            const uint32_t bytes = (uint32_t)(((cnt + kPad - 1) / kPad) * kPad * sizeof(T));
            for (int j = 0; j <= B; ++j) {
                T* dst = estore + (size_t)j * (size_t)P.ld + (size_t)cta_base;
                const uint32_t src = (uint32_t)__cvta_generic_to_shared(e_s + (size_t)j * kPcCta);
                asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                             :: "l"(dst), "r"(src), "r"(bytes) : "memory");
            }
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
    }
}

// Response form of the FP64 predictor-corrector path (polynomial volatility,
// at most kRespDates dates), as path_kernel_fp64_resp in hjm_forward.cu: the
// polynomial parts, whose step with the N-projected loadings is
//     S' = S + c dtau U + (c + c^2) dtau^2 W + aS.phi,  U' = U + 2 c dtau W + aU.phi,
//     W' = W + aW.phi   (old values on the right),
// as double-FP32 sums in the block's moving frame of that step (frame_step,
// frame_block_end in hjm_resp.cuh), and the remainder, driven at L-1 and L by W and by the step's curvature
// noise, as double-FP32 sums of the predictor-corrector response table (the
// coefficient of the old W per date slot and lag; response_table_kernel with
// pc = 1) over the active prefix of slots.  TRI: factor k of degree <= k
// (aU[0] = aW[0] = aW[1] = 0).
template <int NT, bool EXT, bool TRI, bool SC>
__global__ void __launch_bounds__(kPcCta, 6)
    path_kernel_pc_resp(const __grid_constant__ PcParams<double> Q, const float4* __restrict__ resp,
                        const double* __restrict__ ext, double* __restrict__ partials, double* __restrict__ estore)
{
    const PathParams<double>& P = Q.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    double* cf_s = reinterpret_cast<double*>(smem);  // [B+2][kPcCta]; exposures alias it one row up
    double* red_s = cf_s + (size_t)(B + 2) * kPcCta;

    const int64_t cta_base = (int64_t)blockIdx.x * kPcCta;
    const int64_t lp = cta_base + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;

    float2 A[kRespSlots], Al[kRespSlots];  // {remainder at tenor j, its running sum}, slot B - j, hi + lo
#pragma unroll
    for (int r = 0; r < kRespSlots; ++r) A[r] = Al[r] = make_float2(0.0f, 0.0f);
    // the parts S, U, W in the block's moving frame, {y_c, v_c} as hi + lo
    // pairs, and their FP64 running sums between blocks (shared memory)
    float2 Y[3], Yl[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) Y[c] = Yl[c] = make_float2(0.0f, 0.0f);
    double* z_s = red_s + 2 * (kPcCta / 32);
#pragma unroll
    for (int c = 0; c < 3; ++c) z_s[c * kPcCta + tid] = 0.0;
    const BlockFrame F(Q.k1, Q.k2p, Q.k1x2, (double)P.stride);  // the two-stage step on a quadratic
    // the frame's coefficient rows (one block's), staged in shared memory for SC
    const float4* coef = resp + resp_coef_offset(P.stride, B);
    if constexpr (SC) {
        float4* c_s = reinterpret_cast<float4*>(z_s + 3 * kPcCta);
        for (int i = tid; i < P.stride * kStateRow; i += kPcCta) c_s[i] = coef[i];
        __syncthreads();
        coef = c_s;
    }
    // the active prefix of each row, after the table's response and coefficient rows
    const int* nact = reinterpret_cast<const int*>(resp + resp_nact_offset(P.stride, B));

    auto sample = [&](int i) {
        const double tau = P.tau[i];
        const float2 h = select_reg<kRespSlots, float2>(A, B - i), l = select_reg<kRespSlots, float2>(Al, B - i);
        const double hc = widen_f32(h.x) + widen_f32(l.x), hcs = widen_f32(h.y) + widen_f32(l.y);
        double S = 0.0, U = 0.0, W = 0.0, ZS = 0.0, ZU = 0.0, ZW = 0.0;
        if (i >= 2) frame_block_end(Y, Yl, F, z_s + tid, kPcCta, S, U, W, ZS, ZU, ZW);
        const double x = P.psamp[i] + (fma(tau, fma(tau, W, U), S) + hc);
        const double acc = fma(tau, fma(tau, ZW, ZU), ZS) + hcs;
        const double D = exp(-(P.psum[i] + acc) * P.dt);
        const double Lb = P.m * (exp(x * P.inv_m) - 1.0);
        cf_s[i * kPcCta + tid] = D * (P.payA[i] * Lb - P.payB[i]);
    };

    sample(1);
    for (int b = 1; b < B; ++b) {
        const float4* row = resp + (size_t)b * P.stride * kRespRow;
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
            const int n_act = __ldg(nact + n);  // uniform: the row's active prefix
            const float4* rr = row + (size_t)s * kRespRow;
            // the remainder's sources read W before this step's update
            const float2 wh2 = make_float2(Y[2].x, Y[2].x), wl2 = make_float2(Yl[2].x, Yl[2].x);
            const float2 nwh2 = make_float2(-Y[2].x, -Y[2].x);
            resp_groups(n_act, [&](auto gc) {
                constexpr int G = decltype(gc)::value;
                float4 k[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) k[u] = __ldg(rr + 4 * G + u);
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    df_acc(A[4 * G + u], Al[4 * G + u], make_float2(k[u].x, k[u].y), make_float2(k[u].z, k[u].w),
                           wh2, wl2, nwh2);
            });
            frame_step<EXT, TRI, SC>(Y, Yl, coef + (size_t)s * kStateRow, ph, pl);
        }
        sample(b + 1);
    }
    fp64_epilogue<kPcCta>(P, cf_s, cf_s + kPcCta, red_s, partials, estore, cta_base, active);
}

template <int NT, bool EXT, bool TRI>
static cudaError_t launch_pc_resp_t(const PcParams<double>& Q, const float4* resp, const double* ext,
                                    double* partials, double* estore, cudaStream_t s)
{
    // cf_s [B+2][kCta], red_s, the parts' running sums [3][kCta], the frame's coefficients
    const bool sc = Q.P.stride <= kFrameSmemRows;
    const size_t smem = ((size_t)Q.P.n_blocks + 2) * kPcCta * 8 + 2 * (kPcCta / 32) * 8 + 3 * kPcCta * 8 +
                        (sc ? (size_t)Q.P.stride * kStateRow * 16 : 0);
    auto k = sc ? path_kernel_pc_resp<NT, EXT, TRI, true> : path_kernel_pc_resp<NT, EXT, TRI, false>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (Q.P.n_paths + kPcCta - 1) / kPcCta;
    k<<<(unsigned)grid, kPcCta, smem, s>>>(Q, resp, ext, partials, estore);
    return cudaGetLastError();
}

template <int NT>
static cudaError_t launch_pc_resp_nt(const PcParams<double>& Q, const float4* resp, const double* ext,
                                     double* partials, double* estore, cudaStream_t s)
{
    const bool tri = Q.aU[0] == 0.0 && Q.aW[0] == 0.0 && Q.aW[1] == 0.0;
    if (ext) return tri ? launch_pc_resp_t<NT, true, true>(Q, resp, ext, partials, estore, s)
                        : launch_pc_resp_t<NT, true, false>(Q, resp, ext, partials, estore, s);
    return tri ? launch_pc_resp_t<NT, false, true>(Q, resp, ext, partials, estore, s)
               : launch_pc_resp_t<NT, false, false>(Q, resp, ext, partials, estore, s);
}

template <int NT, typename T, bool EXT, bool POLY>
static cudaError_t launch_pc_t(const PcParams<T>& Q, const double* ext, double* partials, T* estore, cudaStream_t s)
{
    const size_t smem = pc_smem_bytes(NT, Q.P.n_blocks, sizeof(T));
    auto k = path_kernel_pc<NT, T, EXT, POLY>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (Q.P.n_paths + kPcCta - 1) / kPcCta;
    k<<<(unsigned)grid, kPcCta, smem, s>>>(Q, ext, partials, estore);
    return cudaGetLastError();
}

template <int NT, typename T>
static cudaError_t launch_pc_nt(const PcParams<T>& Q, bool poly, const double* ext, double* partials, T* estore,
                                cudaStream_t s)
{
    if (ext) return poly ? launch_pc_t<NT, T, true, true>(Q, ext, partials, estore, s)
                         : launch_pc_t<NT, T, true, false>(Q, ext, partials, estore, s);
    return poly ? launch_pc_t<NT, T, false, true>(Q, ext, partials, estore, s)
                : launch_pc_t<NT, T, false, false>(Q, ext, partials, estore, s);
}

template <typename T>
static cudaError_t launch_pc_any(int nt, const PcParams<T>& Q, bool poly, const double* ext, double* partials,
                                 T* estore, cudaStream_t s)
{
    if (nt == 51) return launch_pc_nt<51, T>(Q, poly, ext, partials, estore, s);
    if (nt == 61) return launch_pc_nt<61, T>(Q, poly, ext, partials, estore, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_path_pc(int nt, const PcParams<double>& Q, bool poly, const float4* resp, const double* ext,
                           double* partials, double* estore, cudaStream_t s)
{
    if (resp) {
        if (!poly || Q.P.n_blocks > kRespDates) return cudaErrorInvalidValue;
        if (nt == 51) return launch_pc_resp_nt<51>(Q, resp, ext, partials, estore, s);
        if (nt == 61) return launch_pc_resp_nt<61>(Q, resp, ext, partials, estore, s);
        return cudaErrorInvalidValue;
    }
    return launch_pc_any<double>(nt, Q, poly, ext, partials, estore, s);
}

cudaError_t launch_path_pc(int nt, const PcParams<float>& Q, bool poly, const double* ext, double* partials,
                           float* estore, cudaStream_t s)
{
    return launch_pc_any<float>(nt, Q, poly, ext, partials, estore, s);
}

size_t pc_smem(int nt, int n_blocks, bool mixed) { return pc_smem_bytes(nt, n_blocks, mixed ? 4 : 8); }

int pc_cta() { return kPcCta; }

}  // namespace hjm
