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

cudaError_t launch_path_pc(int nt, const PcParams<double>& Q, bool poly, const double* ext, double* partials,
                           double* estore, cudaStream_t s)
{
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
