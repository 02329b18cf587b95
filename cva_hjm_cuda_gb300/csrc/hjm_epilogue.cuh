// hjm_epilogue.cuh -- the end of the path kernels (FP64: Euler and the
// volatility-table response form in hjm_forward.cu, predictor-corrector in
// hjm_pc.cu, the response forms' windows in hjm_eresp.cu and hjm_forward.cu;
// mixed precision: the convected pairs in hjm_forward.cu): exposures, the
// CTA's partial sums and the exposure store.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

#include "hjm_device.cuh"

namespace hjm {

// Epilogue of the FP64 path kernels: the exposure profile E_j = max(sum_{i>j}
// cf_i, 0) by FP64 suffix sums, the path's CVA contribution sum_j cvaw[j] E_j,
// the CTA's partial sums (dates 0..B, then sum c and sum c^2) and, if asked,
// the exposure rows of the CTA's paths to HBM.  cf_s rows 1..B hold the cash
// flows, column tid private to its thread; e_s (B+1 rows) may alias cf_s one
// row up: row j of e_s is written after row j+1 of cf_s, the one aliased, is read.
template <int kCta>
__device__ __forceinline__ void fp64_epilogue(const PathParams<double>& P, const double* cf_s, double* e_s,
                                              double* red_s, double* __restrict__ partials,
                                              double* __restrict__ estore, int64_t cta_base, bool active)
{
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    double v = 0.0, cva_c = 0.0;
    e_s[B * kCta + tid] = 0.0;
    for (int j = B - 1; j >= 0; --j) {
        v += cf_s[(j + 1) * kCta + tid];
        double e = (v > 0.0) ? v : 0.0;
        if (!active) e = 0.0;
        e_s[j * kCta + tid] = e;
        cva_c = fma(P.cvaw[j], e, cva_c);
    }
    __syncthreads();

    // CTA partial sums: dates 0..B, then sum c and sum c^2
    const int warp = tid >> 5, lane = tid & 31;
    const int R = B + 3;
    for (int j = warp; j <= B; j += kCta / 32) {
        double sum = 0.0;
#pragma unroll
        for (int q = 0; q < kCta / 32; ++q) sum += e_s[j * kCta + lane + 32 * q];
        sum = warp_sum(sum);
        if (lane == 0) partials[(size_t)blockIdx.x * R + j] = sum;
    }
    {
        const double s1 = warp_sum(cva_c), s2 = warp_sum(cva_c * cva_c);
        if (lane == 0) {
            red_s[warp] = s1;
            red_s[kCta / 32 + warp] = s2;
        }
    }
    if (P.store_exposures) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kCta / 32; ++w) {
            s1 += red_s[w];
            s2 += red_s[kCta / 32 + w];
        }
        partials[(size_t)blockIdx.x * R + B + 1] = s1;
        partials[(size_t)blockIdx.x * R + B + 2] = s2;
        if (P.store_exposures) {
            // date rows of this CTA's paths, smem -> HBM with the bulk-copy (TMA) engine
            const int64_t cnt = (P.n_paths - cta_base < kCta) ? (P.n_paths - cta_base) : kCta;
            const uint32_t bytes = (uint32_t)(((cnt + 1) / 2) * 2 * sizeof(double));
            for (int j = 0; j <= B; ++j) {
                double* dst = estore + (size_t)j * (size_t)P.ld + (size_t)cta_base;
                const uint32_t src = (uint32_t)__cvta_generic_to_shared(e_s + (size_t)j * kCta);
                asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                             :: "l"(dst), "r"(src), "r"(bytes) : "memory");
            }
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
    }
}

// Epilogue of the mixed-precision path kernels (as fp64_epilogue, exposures
// and their store in FP32): acc_s rows 1..B hold the cash flows (FP64), e_s
// B+1 FP32 rows (free for this use).
template <typename CF, int kCta = hjm::kCta>
__device__ __forceinline__ void mixed_epilogue(const PathParams<float>& P, const CF* acc_s, float* e_s,
                                               double* red_s, double* __restrict__ partials,
                                               float* __restrict__ estore, int64_t cta_base, bool active)
{
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    double v = 0.0, cva_c = 0.0;
    e_s[B * kCta + tid] = 0.f;
    for (int j = B - 1; j >= 0; --j) {
        v += as_f64(acc_s[(j + 1) * kCta + tid]);
        double e = (v > 0.0) ? v : 0.0;
        if (!active) e = 0.0;
        e_s[j * kCta + tid] = (float)e;
        cva_c = fma(P.cvaw[j], e, cva_c);
    }
    __syncthreads();

    const int warp = tid >> 5, lane = tid & 31;
    const int R = B + 3;
    for (int j = warp; j <= B; j += kCta / 32) {
        double sum = 0.0;
#pragma unroll
        for (int q = 0; q < kCta / 32; ++q) sum += (double)e_s[j * kCta + lane + 32 * q];
        sum = warp_sum(sum);
        if (lane == 0) partials[(size_t)blockIdx.x * R + j] = sum;
    }
    {
        const double s1 = warp_sum(cva_c), s2 = warp_sum(cva_c * cva_c);
        if (lane == 0) {
            red_s[warp] = s1;
            red_s[kCta / 32 + warp] = s2;
        }
    }
    if (P.store_exposures) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kCta / 32; ++w) {
            s1 += red_s[w];
            s2 += red_s[kCta / 32 + w];
        }
        partials[(size_t)blockIdx.x * R + B + 1] = s1;
        partials[(size_t)blockIdx.x * R + B + 2] = s2;
        if (P.store_exposures) {
            const int64_t cnt = (P.n_paths - cta_base < kCta) ? (P.n_paths - cta_base) : kCta;
            const uint32_t bytes = (uint32_t)(((cnt + 3) / 4) * 4 * sizeof(float));
            for (int j = 0; j <= B; ++j) {
                float* dst = estore + (size_t)j * (size_t)P.ld + (size_t)cta_base;
                const uint32_t src = (uint32_t)__cvta_generic_to_shared(e_s + (size_t)j * kCta);
                asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                             :: "l"(dst), "r"(src), "r"(bytes) : "memory");
            }
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
    }
}

// Epilogue of a window: exposures E_j = max(sum_{i > j} cf_i, 0) of dates
// j in [lo - 1, hi - 1] (and E_B = 0 for the latest window), the cash flows of
// later dates arriving in carry; the CTA's EE partial sums of those dates;
// the CVA statistics (sum c, sum c^2 of the per-path contributions) from the
// earliest window; the exposure rows by the bulk-copy engine.
template <int kCta>
__device__ __forceinline__ void window_epilogue(const PathParams<double>& P, int lo, int hi, double* cf_s,
                                                double* red_s, double* __restrict__ partials,
                                                double* __restrict__ estore, double* __restrict__ carry,
                                                int64_t cta_base, int64_t lp, bool active)
{
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const bool top = hi == B, bottom = lo == 1;
    double* e_s = cf_s + kCta;  // exposure row of date j: j - lo + 1 (the cash-flow row of date j + 1)
    double v = 0.0, cva_c = 0.0;
    if (!top && active) {
        v = carry[lp];
        cva_c = carry[P.n_paths + lp];
    }
    if (top) e_s[(size_t)(B - lo + 1) * kCta + tid] = 0.0;
    for (int j = hi - 1; j >= lo - 1; --j) {
        v += cf_s[(size_t)(j - lo + 2) * kCta + tid];
        double e = (v > 0.0) ? v : 0.0;
        if (!active) e = 0.0;
        e_s[(size_t)(j - lo + 1) * kCta + tid] = e;
        cva_c = fma(P.cvaw[j], e, cva_c);
    }
    if (!bottom && active) {
        carry[lp] = v;
        carry[P.n_paths + lp] = cva_c;
    }
    __syncthreads();

    const int warp = tid >> 5, lane = tid & 31;
    const int R = B + 3;
    const int j0 = lo - 1, j1 = top ? B : hi - 1;
    for (int j = j0 + warp; j <= j1; j += kCta / 32) {
        double sum = 0.0;
#pragma unroll
        for (int q = 0; q < kCta / 32; ++q) sum += e_s[(size_t)(j - lo + 1) * kCta + lane + 32 * q];
        sum = warp_sum(sum);
        if (lane == 0) partials[(size_t)blockIdx.x * R + j] = sum;
    }
    if (bottom) {
        const double s1 = warp_sum(cva_c), s2 = warp_sum(cva_c * cva_c);
        if (lane == 0) {
            red_s[warp] = s1;
            red_s[kCta / 32 + warp] = s2;
        }
    }
    if (P.store_exposures) asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
    if (tid == 0) {
        if (bottom) {
            double s1 = 0.0, s2 = 0.0;
            for (int w = 0; w < kCta / 32; ++w) {
                s1 += red_s[w];
                s2 += red_s[kCta / 32 + w];
            }
            partials[(size_t)blockIdx.x * R + B + 1] = s1;
            partials[(size_t)blockIdx.x * R + B + 2] = s2;
        }
        if (P.store_exposures) {
            // date rows of this CTA's paths, smem -> HBM with the bulk-copy (TMA) engine
            const int64_t cnt = (P.n_paths - cta_base < kCta) ? (P.n_paths - cta_base) : kCta;
            const uint32_t bytes = (uint32_t)(((cnt + 1) / 2) * 2 * sizeof(double));
            for (int j = j0; j <= j1; ++j) {
                double* dst = estore + (size_t)j * (size_t)P.ld + (size_t)cta_base;
                const uint32_t src = (uint32_t)__cvta_generic_to_shared(e_s + (size_t)(j - lo + 1) * kCta);
                asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                             :: "l"(dst), "r"(src), "r"(bytes) : "memory");
            }
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
    }
}

}  // namespace hjm
