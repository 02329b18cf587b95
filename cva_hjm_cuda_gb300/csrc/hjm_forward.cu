// hjm_forward.cu -- fused Monte Carlo path kernel, reductions and PFE selection.
//
// One launch of path_kernel replaces the reference's whole GPU pipeline
// (simulation_gpu.cu:956-1179): cuRAND normal buffer (:1057-1071), 2,500
// single-step launches each followed by cudaDeviceSynchronize (:724-796, or
// the 50-step kernel4 variant :471-669), the exposure kernel (:803-882) and
// the cuBLAS gemv column sum (:889-933).  One thread owns one Monte Carlo
// path for its whole life: the curve sits in registers, normals come from
// Philox in registers, the numeraire of each 0.5y block end is priced on the
// spot, and the per-path exposure profile is reduced inside the CTA.
//
// Semantics follow the reference CPU path (simulation_cpu.h:188-296), which
// the reference's shared-memory GPU kernel also reproduces (xls RMSE 0.0):
//   * block 0 (steps 0..stride-1) holds the curve at spot (simulation_cpu.h:212);
//   * after block b the numeraire of tenor i = b+1 is sampled: forward f[i] and
//     discount exp(-dt * sum of f[i] over all steps so far) (simulation_cpu.h:248-250);
//   * cash flow of date i: D_i * N * alpha_i * (L_i - K), L = m (e^{f/m} - 1);
//     exposure E_j = max(sum_{i>j} cf_i, 0) (simulation_cpu.h:279-295).
#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>

#include "hjm_device.cuh"
#include "hjm_kernels.h"
#include "hjm_pairs.cuh"

namespace hjm {

template <typename T>
struct Prec;
template <>
struct Prec<double> {
    static constexpr bool kMixed = false;
    static constexpr int kThreads = 64;   // FP64: more shared memory per path, fewer paths per CTA
};
template <>
struct Prec<float> {
    static constexpr bool kMixed = true;
    static constexpr int kThreads = kCta;
};

// Shared-memory layout of path_kernel (dynamic), per CTA of kCta threads,
// column tid private to its thread until the epilogue:
//   cf_s   [B+1][kCta] T       cash flows of the sampled dates
//   acc_s  [B+1][kCta] double  FP64 discount sums of the stochastic part per tenor
//   work_s mixed: [max(NT, B+1)][kCta] float   block-partial staging, then exposures
//          FP64:  [2(B+2)][kCta] double        curve at block start / end, then exposures
//   red_s  [2 * kCta/32] double CVA statistics
__host__ __device__ inline int path_threads(bool mixed) { return mixed ? Prec<float>::kThreads : Prec<double>::kThreads; }

__host__ __device__ inline size_t path_smem_bytes(int nt, int n_blocks, bool mixed)
{
    const size_t kCta = (size_t)path_threads(mixed);
    const size_t te = mixed ? 4 : 8;
    const size_t rows = (size_t)n_blocks + 1;
    size_t b = rows * kCta * te;                       // cf_s
    b = (b + 7) & ~(size_t)7;
    b += rows * kCta * 8;                              // acc_s
    const size_t wrows = mixed ? ((size_t)nt > rows ? (size_t)nt : rows) : 2 * (rows + 1);
    b = (b + 127) & ~(size_t)127;
    b += wrows * kCta * te;                            // work_s
    b += 2 * (kCta / 32) * 8;                          // red_s
    return b;
}

// FP64 mode: discount sums by block-sum recovery.  Over one block of Euler
// steps n = n0 .. n0+stride-1 the states h_n = A h_{n-1} + S phi_n sum to
//     (I - A) H = S Phi - A (h_end - h_start),   H = sum_n h_n, Phi = sum_n phi_n,
// and (I - A) H [t] = c (H[t] - H[t+1]) for t below the last tenor.  So with
// one tenor accumulated directly (H[B], the last tenor still to be sampled),
//     H[t] = H[t+1] + (sum_k sv[k][t] Phi_k - (A d)[t]) / c,  d = h_end - h_start,
// gives every block sum the discount needs in O(B) FP64 operations per block
// instead of one FP64 addition per tenor per step (the FP64 pipe is the bound).
// Exact in exact arithmetic; in FP64 the recovered sums differ from step-by-
// step accumulation by ~1e-14 relative.
template <int NT, typename T, bool EXT>
__global__ void __launch_bounds__(Prec<T>::kThreads, Prec<T>::kMixed ? 3 : 4)
    path_kernel(const __grid_constant__ PathParams<T> P, const double* __restrict__ ext,
                double* __restrict__ partials, T* __restrict__ estore)
{
    constexpr bool kMixed = Prec<T>::kMixed;
    constexpr int kCta = Prec<T>::kThreads;  // paths per CTA
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const int rows = B + 1;
    T* cf_s = reinterpret_cast<T*>(smem);
    size_t off = ((size_t)rows * kCta * sizeof(T) + 7) & ~(size_t)7;
    double* acc_s = reinterpret_cast<double*>(smem + off);
    off += (size_t)rows * kCta * 8;
    off = (off + 127) & ~(size_t)127;
    T* work_s = reinterpret_cast<T*>(smem + off);
    const int wrows = kMixed ? (NT > rows ? NT : rows) : 2 * (rows + 1);
    double* red_s = reinterpret_cast<double*>(smem + off + (size_t)wrows * kCta * sizeof(T));

    const int64_t cta_base = (int64_t)blockIdx.x * kCta;
    const int64_t lp = cta_base + tid;            // path index within this launch
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;

    // stochastic part of the curve; zero through block 0 (spot hold)
    T h[NT];
#pragma unroll
    for (int t = 0; t < NT; ++t) h[t] = T(0);
    for (int i = 0; i < rows; ++i) acc_s[i * kCta + tid] = 0.0;

    // mixed: FP32 block partials of the discount sums, folded into acc_s per block
    T pb[kMixed ? NT : 1];
#pragma unroll
    for (int t = 0; t < (kMixed ? NT : 1); ++t) pb[t] = T(0);
    // FP64: curve at the start / end of the block, tenors 0 .. B+1
    double* hs_s = reinterpret_cast<double*>(work_s);
    double* he_s = hs_s + (size_t)(rows + 1) * kCta;
    if (!kMixed)
        for (int t = 0; t <= B + 1; ++t) hs_s[t * kCta + tid] = 0.0;

    // price date i from the sampled numeraire (x_i, D_i)
    auto sample = [&](int i) {
        const T hi = select_reg<NT, T>(h, i);
        const double x = P.psamp[i] + (double)hi;
        const double a = P.psum[i] + acc_s[i * kCta + tid];
        T cf;
        if constexpr (kMixed) {
            const float D = expf((float)(-a * P.dt));
            const float mm = (float)P.m;
            const float L = mm * expm1f((float)x / mm);
            cf = D * ((float)P.payA[i] * L - (float)P.payB[i]);
        } else {
            const double D = exp(-a * P.dt);
            const double L = P.m * (exp(x / P.m) - 1.0);
            cf = D * (P.payA[i] * L - P.payB[i]);
        }
        cf_s[i * kCta + tid] = cf;
    };

    sample(1);
    const T c = P.c;
    for (int b = 1; b < B; ++b) {
        double f0 = 0.0, f1 = 0.0, f2 = 0.0, hb = 0.0;  // FP64 mode: block sums of phi_k and of h[B]
        for (int s = 0; s < P.stride; ++s) {
            const int n = b * P.stride + s;
            T phi0, phi1, phi2;
            draw_phi<T, EXT>(ext, gpath, active ? lp : 0, P.n_paths, n, P.rk0, P.rk1, phi0, phi1, phi2);
            euler_step<NT, T>(h, P, c, phi0, phi1, phi2);
            if constexpr (kMixed) {
                // only the groups of 8 tenors that meet (b, B] (uniform branches)
#pragma unroll
                for (int g = 0; g < NT; g += 8) {
                    if (g + 7 > b && g <= B) {
#pragma unroll
                        for (int t = (g == 0 ? 1 : g); t < g + 8 && t < NT; ++t) pb[t] += h[t];
                    }
                }
            } else {
                f0 += (double)phi0;
                f1 += (double)phi1;
                f2 += (double)phi2;
                hb += (double)select_reg<NT, T>(h, B);
            }
        }
        if constexpr (kMixed) {
            // fold the FP32 block partials of the tenors still to be sampled
            // into the FP64 accumulators
#pragma unroll
            for (int t = 1; t < NT; ++t) {
                work_s[t * kCta + tid] = pb[t];
                pb[t] = T(0);
            }
            for (int t = b + 1; t <= B; ++t) acc_s[t * kCta + tid] += (double)work_s[t * kCta + tid];
        } else {
            // stage the block-end curve, then recover the block sums of tenors (b, B]
#pragma unroll
            for (int t = 0; t < NT; ++t)
                if (t <= B + 1) he_s[t * kCta + tid] = (double)h[t];
            double Hn = hb;
            acc_s[B * kCta + tid] += Hn;
            double dn = he_s[B * kCta + tid] - hs_s[B * kCta + tid];
            for (int t = B - 1; t > b; --t) {
                const double d = he_s[t * kCta + tid] - hs_s[t * kCta + tid];
                const double xi = fma((double)P.sv[2][t], f2, fma((double)P.sv[1][t], f1, (double)P.sv[0][t] * f0));
                const double ad = fma((double)c, dn - d, d);
                Hn = fma(xi - ad, P.inv_c, Hn);
                acc_s[t * kCta + tid] += Hn;
                dn = d;
            }
            double* tmp = hs_s;
            hs_s = he_s;
            he_s = tmp;
        }
        sample(b + 1);
    }

    // exposure profile E_j = max(sum_{i>j} cf_i, 0), FP64 suffix sums, and the
    // path's CVA contribution sum_j cvaw[j] E_j
    T* e_s = work_s;
    double v = 0.0, cva_c = 0.0;
    e_s[B * kCta + tid] = T(0);
    for (int j = B - 1; j >= 0; --j) {
        v += (double)cf_s[(j + 1) * kCta + tid];
        double e = (v > 0.0) ? v : 0.0;
        if (!active) e = 0.0;
        e_s[j * kCta + tid] = (T)e;
        cva_c = fma(P.cvaw[j], e, cva_c);
    }
    __syncthreads();

    // CTA partial sums: dates 0..B, then sum c and sum c^2
    const int warp = tid >> 5, lane = tid & 31;
    const int R = B + 3;
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
    if (P.store_exposures) {
        // date rows of this CTA's paths, smem -> HBM with the bulk-copy (TMA) engine
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
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
        if (P.store_exposures) {
            const int64_t cnt = (P.n_paths - cta_base < kCta) ? (P.n_paths - cta_base) : kCta;
            constexpr int kVec = 16 / (int)sizeof(T);
            const uint32_t bytes = (uint32_t)(((cnt + kVec - 1) / kVec) * kVec * sizeof(T));
            for (int j = 0; j <= B; ++j) {
                T* dst = estore + (size_t)j * (size_t)P.ld + (size_t)cta_base;
                const uint32_t src = (uint32_t)__cvta_generic_to_shared(e_s + (size_t)j * kCta);
                asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;"
                             :: "l"(dst), "r"(src), "r"(bytes) : "memory");
            }
            asm volatile("cp.async.bulk.commit_group;" ::: "memory");
            asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory");
        }
    }
}

// ---------------------------------------------------------------------------
// Mixed precision with packed FP32x2 arithmetic.  The curve of one path is held
// as H = ceil(NT/2) float2 pairs, pair p = {h[p], h[p+H]}: the upwind neighbour
// h[t+1] of every tenor lies in the same component of pair p+1, so each packed
// FMA (__ffma2_rn) advances two tenors and the Euler step costs half the issue
// slots of the scalar form.  Only the seam pair (p = H-1, whose .x neighbour is
// pair 0's .y), the pair holding the last tenor (backward difference) and the
// padding tenor of an odd grid take scalar fix-ups.  Every element sees exactly
// the scalar kernel's operations (fma(sv, phi, h) three times, one rounded
// difference, fma(c, d, x)), so the results are bit-identical to it.
// ---------------------------------------------------------------------------
// Mixed-precision discount sums: FP32 block sums by the same recovery as the
// FP64 kernel, but anchored at tenor 1 and run upwards,
//     H[t+1] = H[t] - (sum_k sv[k][t] Phi_k - (A d)[t]) / c,   t = 1 .. B-1,
// so a block costs O(B) scalar FP32 operations and four additions per step
// (Phi_k and H[1]) instead of an addition per tenor per step; the FP32 block
// sums are then folded into FP64 per tenor.  The recovered sums differ from
// step-by-step FP32 accumulation by ~1e-6 relative (the FP32 rounding of the
// Euler steps divided by c), far inside the mixed-precision tolerance.
//
// Shared memory per thread: acc (B+1) FP64 discount sums, whose slot i holds
// date i's cash flow once tenor i is sampled; hs (B+2) FP32 curve at the block
// start, reused for the exposure tile at the end.
template <int NT, bool EXT>
__global__ void __launch_bounds__(kCta, 4)
    path_kernel_mixed(const __grid_constant__ MixedParams M, const double* __restrict__ ext,
                      double* __restrict__ partials, float* __restrict__ estore)
{
    constexpr int H = PairGrid<NT>::H;
    const PathParams<float>& P = M.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = P.n_blocks;
    const int rows = B + 1;
    double* acc_s = reinterpret_cast<double*>(smem);                       // [B+1][kCta]
    float* hs_s = reinterpret_cast<float*>(smem + (size_t)rows * kCta * 8);  // [B+2][kCta]
    double* red_s = reinterpret_cast<double*>(smem + (size_t)rows * kCta * 8 + (size_t)(rows + 1) * kCta * 4);

    const int64_t cta_base = (int64_t)blockIdx.x * kCta;
    const int64_t lp = cta_base + tid;
    const bool active = lp < P.n_paths;
    const uint64_t gpath = P.path_offset + (uint64_t)lp;

    float2 h[H];
#pragma unroll
    for (int p = 0; p < H; ++p) h[p] = make_float2(0.f, 0.f);
    for (int i = 0; i < rows; ++i) acc_s[i * kCta + tid] = 0.0;
    for (int t = 0; t <= B + 1; ++t) hs_s[t * kCta + tid] = 0.f;

    // tenor t of the packed curve (t static after unrolling)
    auto ht = [&](int t) -> float { return t < H ? h[t].x : h[t - H].y; };

    auto sample = [&](int i) {
        const double x = P.psamp[i] + (double)select_pair<NT>(h, i);
        const double a = P.psum[i] + acc_s[i * kCta + tid];
        const float D = expf((float)(-a * P.dt));
        const float mm = (float)P.m;
        const float L = mm * expm1f((float)x / mm);
        acc_s[i * kCta + tid] = (double)(D * ((float)P.payA[i] * L - (float)P.payB[i]));  // cash flow of date i
    };

    sample(1);
    for (int b = 1; b < B; ++b) {
        float F0 = 0.f, F1 = 0.f, F2 = 0.f, H1 = 0.f;  // block sums of phi_k and of h[1]
        for (int s = 0; s < P.stride; ++s) {
            const int n = b * P.stride + s;
            float phi0, phi1, phi2;
            draw_phi<float, EXT>(ext, gpath, active ? lp : 0, P.n_paths, n, P.rk0, P.rk1, phi0, phi1, phi2);
            euler_step_pairs<NT>(h, M, phi0, phi1, phi2);
            F0 += phi0;
            F1 += phi1;
            F2 += phi2;
            H1 += h[1].x;
        }
        // recover the block sums of tenors 2 .. B upwards from H[1]; fold (b, B] into FP64
        recover_sums_up<NT>(h, hs_s, tid, kCta, P, F0, F1, F2, H1, B, [&](int t, float Ht) {
            if (t > b) acc_s[t * kCta + tid] += (double)Ht;
        });
        // the block-end curve is the next block's start (tenors 1 .. B+1)
#pragma unroll
        for (int t = 1; t < NT; ++t)
            if (t <= B + 1) hs_s[t * kCta + tid] = ht(t);
        sample(b + 1);
    }

    float* e_s = hs_s;  // [B+1][kCta] exposures
    double v = 0.0, cva_c = 0.0;
    e_s[B * kCta + tid] = 0.f;
    for (int j = B - 1; j >= 0; --j) {
        v += acc_s[(j + 1) * kCta + tid];
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

__host__ __device__ inline size_t mixed_smem_bytes(int nt, int n_blocks)
{
    (void)nt;
    const size_t rows = (size_t)n_blocks + 1;
    return rows * kCta * 8 + (rows + 1) * kCta * 4 + 2 * (kCta / 32) * 8;
}

void pack_mixed_params(int nt, const PathParams<float>& P, MixedParams& M)
{
    std::memset(&M, 0, sizeof(M));
    M.P = P;
    const int H = (nt + 1) / 2;
    for (int k = 0; k < kFactors; ++k)
        for (int p = 0; p < H; ++p) {
            M.svp[k][p].x = P.sv[k][p];
            M.svp[k][p].y = (H + p < nt) ? P.sv[k][H + p] : 0.0f;
        }
    M.cp = make_float2(P.c, P.c);
}

// ---------------------------------------------------------------------------
// Deterministic column sums of the CTA partials (Neumaier-compensated FP64):
// one CTA per column, fixed assignment of rows to threads, fixed tree order.
// Replaces the cuBLAS gemv with a ones vector (simulation_gpu.cu:889-933) and
// the host vAdd/saxpy (simulation_gpu.cu:941-951, 1157-1179).
// ---------------------------------------------------------------------------
constexpr int kReduceThreads = 256;

__device__ __forceinline__ void neumaier_add(double& s, double& comp, double x)
{
    const double t = s + x;
    comp += (fabs(s) >= fabs(x)) ? ((s - t) + x) : ((x - t) + s);
    s = t;
}

__global__ void __launch_bounds__(kReduceThreads)
    reduce_columns(const double* __restrict__ partials, int64_t n_rows, int R, double* __restrict__ sums)
{
    __shared__ double ss[kReduceThreads], cs[kReduceThreads];
    const int col = blockIdx.x;
    double s = 0.0, comp = 0.0;
    for (int64_t r = threadIdx.x; r < n_rows; r += kReduceThreads) neumaier_add(s, comp, partials[(size_t)r * R + col]);
    ss[threadIdx.x] = s;
    cs[threadIdx.x] = comp;
    __syncthreads();
    for (int w = kReduceThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            double a = ss[threadIdx.x], ca = cs[threadIdx.x] + cs[threadIdx.x + w];
            neumaier_add(a, ca, ss[threadIdx.x + w]);
            ss[threadIdx.x] = a;
            cs[threadIdx.x] = ca;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) sums[col] = ss[0] + cs[0];
}

// EE, CVA, its standard error and dCVA/dhazard from the column sums.
__global__ void finalize_results(const double* __restrict__ sums, FinalParams F, double* __restrict__ result)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int B = F.n_blocks;
    const double inv_n = 1.0 / (double)F.n_paths;
    double cva = 0.0, dcva = 0.0;
    for (int j = 0; j < kMaxTenor; ++j) {
        const double ee = (j <= B) ? sums[j] * inv_n : 0.0;
        result[kResEE + j] = ee;
        cva += F.cvaw[j] * ee;
        dcva += F.dcvaw[j] * ee;
    }
    const double s1 = sums[B + 1], s2 = sums[B + 2];
    const double n = (double)F.n_paths;
    const double var = (n > 1.0) ? fmax((s2 - s1 * s1 / n) / (n - 1.0), 0.0) : 0.0;
    result[kResCVA] = cva;
    result[kResCVAStderr] = sqrt(var / n);
    result[kResDCVADHazard] = dcva;
    result[kResCVAPathMean] = s1 * inv_n;
}

// ---------------------------------------------------------------------------
// PFE: exact k-th smallest exposure of every date column by most-significant-
// digit radix selection on the IEEE bit patterns (exposures are >= +0, so the
// unsigned order of the bits is the numeric order).  8-bit digits; each pass
// histograms the candidates that match the prefix found so far.
// ---------------------------------------------------------------------------
template <typename K>
__global__ void pfe_hist(const K* __restrict__ keys, int64_t ld, int64_t n, const SelState* __restrict__ st,
                         uint32_t* __restrict__ hist, int shift)
{
    __shared__ uint32_t h[256];
    const int date = blockIdx.y;
    for (int i = threadIdx.x; i < 256; i += blockDim.x) h[i] = 0;
    __syncthreads();
    const uint64_t prefix = st[date].prefix, mask = st[date].mask;
    const K* col = keys + (size_t)date * (size_t)ld;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride) {
        const int64_t i = base + threadIdx.x;
        bool take = false;
        uint32_t digit = 0;
        if (i < n) {
            const uint64_t k = (uint64_t)col[i];
            take = (k & mask) == prefix;
            digit = (uint32_t)(k >> shift) & 0xFFu;
        }
        // warp-aggregated increments: one atomic per distinct digit per warp
        const uint32_t active = __ballot_sync(0xffffffffu, take);
        if (take) {
            const uint32_t peers = __match_any_sync(active, digit);
            if ((threadIdx.x & 31) == (__ffs(peers) - 1)) atomicAdd(&h[digit], (uint32_t)__popc(peers));
        }
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[date * 256 + i], h[i]);
}

__global__ void pfe_scan(SelState* __restrict__ st, uint32_t* __restrict__ hist, int shift)
{
    const int date = blockIdx.x;
    if (threadIdx.x == 0) {
        uint64_t k = st[date].k;
        uint32_t* hd = hist + date * 256;
        int d = 0;
        for (; d < 255; ++d) {
            if (k < hd[d]) break;
            k -= hd[d];
        }
        st[date].prefix |= (uint64_t)d << shift;
        st[date].mask |= (uint64_t)0xFF << shift;
        st[date].k = k;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 256; i += blockDim.x) hist[date * 256 + i] = 0;
}

template <typename K>
__global__ void pfe_write(const SelState* __restrict__ st, int n_dates, double* __restrict__ result)
{
    const int j = threadIdx.x;
    if (j < kMaxTenor) {
        double v = 0.0;
        if (j < n_dates) {
            if (sizeof(K) == 8) {
                v = __longlong_as_double((long long)st[j].prefix);
            } else {
                v = (double)__uint_as_float((uint32_t)st[j].prefix);
            }
        }
        result[kResPFE + j] = v;
    }
}

__global__ void pfe_init(SelState* __restrict__ st, int n_dates, uint64_t k0)
{
    const int j = threadIdx.x;
    if (j < n_dates) {
        st[j].prefix = 0;
        st[j].mask = 0;
        st[j].k = k0;
    }
}

// ---------------------------------------------------------------------------
// Diagnostics: the device's normals and raw Philox words; layout transposes.
// ---------------------------------------------------------------------------
__global__ void dump_normals_kernel(int64_t n_paths, uint64_t path_offset, int n_steps, uint32_t k0, uint32_t k1,
                                    double* __restrict__ out)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n_paths * (int64_t)n_steps) return;
    const int64_t p = idx / n_steps;
    const int n = (int)(idx % n_steps);
    const uint4 w = philox4x32_10(normals_counter(path_offset + (uint64_t)p, (uint32_t)n), k0, k1);
    float z0, z1, z2;
    normals3(w, z0, z1, z2);
    out[idx * 3 + 0] = (double)z0;
    out[idx * 3 + 1] = (double)z1;
    out[idx * 3 + 2] = (double)z2;
}

__global__ void philox_words_kernel(int64_t n_paths, uint64_t path_offset, uint32_t step, uint32_t k0, uint32_t k1,
                                    uint32_t* __restrict__ out)
{
    const int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_paths) return;
    const uint4 w = philox4x32_10(normals_counter(path_offset + (uint64_t)p, step), k0, k1);
    out[p * 4 + 0] = w.x;
    out[p * 4 + 1] = w.y;
    out[p * 4 + 2] = w.z;
    out[p * 4 + 3] = w.w;
}

// [path][step][3] -> [step][3][path] so that the path kernel reads coalesced
__global__ void transpose_normals_kernel(const double* __restrict__ in, int64_t n_paths, int n_steps,
                                         double* __restrict__ out)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t total = n_paths * (int64_t)n_steps * 3;
    if (idx >= total) return;
    const int64_t p = idx % n_paths;
    const int64_t rest = idx / n_paths;  // = n * 3 + k
    out[idx] = in[(size_t)p * n_steps * 3 + (size_t)rest];
}

// [date][ld] of T -> [date][n_paths] of double
template <typename T>
__global__ void widen_exposures_kernel(const T* __restrict__ in, int64_t ld, int64_t n_paths, int n_dates,
                                       double* __restrict__ out)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= n_paths * (int64_t)n_dates) return;
    const int64_t j = idx / n_paths, p = idx % n_paths;
    out[idx] = (double)in[(size_t)j * ld + p];
}

// ---------------------------------------------------------------------------
// Host launchers
// ---------------------------------------------------------------------------
template <int NT, typename T, bool EXT>
static cudaError_t launch_path_t(const PathParams<T>& P, const double* ext, double* partials, T* estore,
                                 cudaStream_t s)
{
    const size_t smem = path_smem_bytes(NT, P.n_blocks, Prec<T>::kMixed);
    auto k = path_kernel<NT, T, EXT>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    constexpr int cta = Prec<T>::kThreads;
    const int64_t grid = (P.n_paths + cta - 1) / cta;
    k<<<(unsigned)grid, cta, smem, s>>>(P, ext, partials, estore);
    return cudaGetLastError();
}

template <typename T>
static cudaError_t launch_path_nt(int nt, const PathParams<T>& P, const double* ext, double* partials, T* estore,
                                  cudaStream_t s)
{
    if (nt == 51) return ext ? launch_path_t<51, T, true>(P, ext, partials, estore, s)
                             : launch_path_t<51, T, false>(P, ext, partials, estore, s);
    if (nt == 61) return ext ? launch_path_t<61, T, true>(P, ext, partials, estore, s)
                             : launch_path_t<61, T, false>(P, ext, partials, estore, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_path_fp64(int nt, const PathParams<double>& P, const double* ext, double* partials,
                             double* estore, cudaStream_t s)
{
    return launch_path_nt<double>(nt, P, ext, partials, estore, s);
}

template <int NT, bool EXT>
static cudaError_t launch_mixed_t(const MixedParams& M, const double* ext, double* partials, float* estore,
                                  cudaStream_t s)
{
    const size_t smem = mixed_smem_bytes(NT, M.P.n_blocks);
    auto k = path_kernel_mixed<NT, EXT>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (M.P.n_paths + kCta - 1) / kCta;
    k<<<(unsigned)grid, kCta, smem, s>>>(M, ext, partials, estore);
    return cudaGetLastError();
}

cudaError_t launch_path_mixed(int nt, const MixedParams& M, const double* ext, double* partials, float* estore,
                              cudaStream_t s)
{
    if (nt == 51) return ext ? launch_mixed_t<51, true>(M, ext, partials, estore, s)
                             : launch_mixed_t<51, false>(M, ext, partials, estore, s);
    if (nt == 61) return ext ? launch_mixed_t<61, true>(M, ext, partials, estore, s)
                             : launch_mixed_t<61, false>(M, ext, partials, estore, s);
    return cudaErrorInvalidValue;
}

bool path_tenor_supported(int nt) { return nt == 51 || nt == 61; }

size_t path_smem(int nt, int n_blocks, bool mixed)
{
    return mixed ? mixed_smem_bytes(nt, n_blocks) : path_smem_bytes(nt, n_blocks, false);
}

int path_cta(bool mixed) { return path_threads(mixed); }

cudaError_t launch_reduce(const double* partials, int64_t n_rows, int R, double* sums, const FinalParams& F,
                          double* result, cudaStream_t s)
{
    reduce_columns<<<R, kReduceThreads, 0, s>>>(partials, n_rows, R, sums);
    finalize_results<<<1, 32, 0, s>>>(sums, F, result);
    return cudaGetLastError();
}

cudaError_t launch_pfe(const void* estore, bool fp64_keys, int64_t ld, int64_t n_paths, int n_dates, uint64_t k0,
                       SelState* st, uint32_t* hist, double* result, int n_sms, cudaStream_t s)
{
    pfe_init<<<1, kMaxTenor, 0, s>>>(st, n_dates, k0);
    cudaMemsetAsync(hist, 0, sizeof(uint32_t) * 256 * (size_t)n_dates, s);
    int64_t gx = (n_paths + 1023) / 1024;
    const int64_t cap = (int64_t)n_sms * 8;
    if (gx > cap) gx = cap;
    if (gx < 1) gx = 1;
    const dim3 grid((unsigned)gx, (unsigned)n_dates);
    const int bits = fp64_keys ? 64 : 32;
    for (int shift = bits - 8; shift >= 0; shift -= 8) {
        if (fp64_keys)
            pfe_hist<uint64_t><<<grid, 256, 0, s>>>((const uint64_t*)estore, ld, n_paths, st, hist, shift);
        else
            pfe_hist<uint32_t><<<grid, 256, 0, s>>>((const uint32_t*)estore, ld, n_paths, st, hist, shift);
        pfe_scan<<<n_dates, 256, 0, s>>>(st, hist, shift);
    }
    if (fp64_keys)
        pfe_write<uint64_t><<<1, kMaxTenor, 0, s>>>(st, n_dates, result);
    else
        pfe_write<uint32_t><<<1, kMaxTenor, 0, s>>>(st, n_dates, result);
    return cudaGetLastError();
}

cudaError_t launch_dump_normals(int64_t n_paths, uint64_t path_offset, int n_steps, uint32_t k0, uint32_t k1,
                                double* out, cudaStream_t s)
{
    const int64_t total = n_paths * (int64_t)n_steps;
    dump_normals_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(n_paths, path_offset, n_steps, k0, k1, out);
    return cudaGetLastError();
}

cudaError_t launch_philox_words(int64_t n_paths, uint64_t path_offset, uint32_t step, uint32_t k0, uint32_t k1,
                                uint32_t* out, cudaStream_t s)
{
    philox_words_kernel<<<(unsigned)((n_paths + 255) / 256), 256, 0, s>>>(n_paths, path_offset, step, k0, k1, out);
    return cudaGetLastError();
}

cudaError_t launch_transpose_normals(const double* in, int64_t n_paths, int n_steps, double* out, cudaStream_t s)
{
    const int64_t total = n_paths * (int64_t)n_steps * 3;
    transpose_normals_kernel<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(in, n_paths, n_steps, out);
    return cudaGetLastError();
}

cudaError_t launch_widen_exposures(const void* in, bool fp64, int64_t ld, int64_t n_paths, int n_dates, double* out,
                                   cudaStream_t s)
{
    const int64_t total = n_paths * (int64_t)n_dates;
    const unsigned g = (unsigned)((total + 255) / 256);
    if (fp64)
        widen_exposures_kernel<double><<<g, 256, 0, s>>>((const double*)in, ld, n_paths, n_dates, out);
    else
        widen_exposures_kernel<float><<<g, 256, 0, s>>>((const float*)in, ld, n_paths, n_dates, out);
    return cudaGetLastError();
}

}  // namespace hjm
