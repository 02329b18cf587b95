// hjm_mlmc.cu -- the coupled level kernel of the multi-level Monte Carlo
// estimator (the reference's doc/TODO:15 lists multi-level MC; new work).
//
// Level l refines the Euler step of level 0 by 2^l.  E[P_L] = E[P_0] +
// sum_{l>=1} E[P_l - P_{l-1}], each correction estimated on its own paths
// with the fine and the coarse curve driven by the same Brownian increments:
// the coarse step's normal is (phi_a + phi_b) / sqrt(2) of the fine steps it
// spans.  One thread evolves both curves of one path (packed FP32x2,
// mixed precision, exactly the arithmetic of path_kernel_mixed for each) and
// the kernel writes the CTA sums of the exposure differences per date and of
// the path's CVA-contribution difference and its square -- the partial-sum
// layout of the valuation, so the same reduction and finalisation give the
// level's EE difference, CVA difference and its standard error.
#include <cuda_runtime.h>

#include <cstdint>

#include "hjm_device.cuh"
#include "hjm_kernels.h"
#include "hjm_pairs.cuh"
#include "hjm_pc.cuh"

namespace hjm {

constexpr int kMlCta = 64;

// Shared memory per thread (columns of kMlCta): accF, accC (B+1) FP64 discount
// sums then cash flows of the fine and coarse curve; hsF, hsC (B+2) FP32
// block-start curves, reused as the FP64 exposure-difference tile.
__host__ __device__ inline size_t mlmc_smem_bytes(int n_blocks)
{
    const size_t rows = (size_t)n_blocks + 1;
    return 2 * rows * kMlCta * 8 + 2 * (rows + 1) * kMlCta * 4 + 2 * (kMlCta / 32) * 8;
}

// Two packed curves per thread: the decomposed form fits 6 CTAs per SM (168
// registers), the table form (three loadings per tenor pair) needs 4.
template <bool POLY>
constexpr int mlmc_min_ctas() { return POLY ? 6 : 4; }

template <int NT, bool POLY>
__global__ void __launch_bounds__(kMlCta, mlmc_min_ctas<POLY>())
    mlmc_level_kernel(const __grid_constant__ MlmcParams Q, double* __restrict__ partials)
{
    const MixedParams& MF = Q.fine;
    const MixedParams& MC = Q.coarse;
    const PathParams<float>& PF = MF.P;
    const PathParams<float>& PC = MC.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = PF.n_blocks;
    const int rows = B + 1;
    double* accF = reinterpret_cast<double*>(smem);
    double* accC = accF + (size_t)rows * kMlCta;
    float* hsF = reinterpret_cast<float*>(accC + (size_t)rows * kMlCta);
    float* hsC = hsF + (size_t)(rows + 1) * kMlCta;
    double* red_s = reinterpret_cast<double*>(hsC + (size_t)(rows + 1) * kMlCta);

    const int64_t cta_base = (int64_t)blockIdx.x * kMlCta;
    const int64_t lp = cta_base + tid;
    const bool active = lp < PF.n_paths;
    const uint64_t gpath = PF.path_offset + (uint64_t)lp;

    MixedPath<NT, POLY> xf, xc;
    xf.reset();
    xc.reset();
    for (int i = 0; i < rows; ++i) {
        accF[i * kMlCta + tid] = 0.0;
        accC[i * kMlCta + tid] = 0.0;
    }
    for (int t = 0; t <= B + 1; ++t) {
        hsF[t * kMlCta + tid] = 0.f;
        hsC[t * kMlCta + tid] = 0.f;
    }
    auto sample = [&](const MixedPath<NT, POLY>& x, const PathParams<float>& P, double* acc, int i) {
        const double xv = P.psamp[i] + (double)x.value(P, i);
        const double a = P.psum[i] + acc[i * kMlCta + tid];
        const float D = expf((float)(-a * P.dt));
        const float mm = (float)P.m;
        const float L = mm * expm1f((float)xv / mm);
        acc[i * kMlCta + tid] = (double)(D * ((float)P.payA[i] * L - (float)P.payB[i]));
    };

    const float kInvSqrt2 = 0.70710678118654752f;
    sample(xf, PF, accF, 1);
    sample(xc, PC, accC, 1);
    for (int b = 1; b < B; ++b) {
        BlockSums bf, bc;
        bf.reset();
        bc.reset();
        xf.begin_block(PF, b);
        xc.begin_block(PC, b);
        for (int k = 0; k < PC.stride; ++k) {
            const int n = b * PF.stride + 2 * k;  // the fine steps n, n+1 make coarse step b*stride_c + k
            float a0, a1, a2, b0, b1, b2;
            draw_phi<float, false>(nullptr, gpath, lp, PF.n_paths, n, PF.rk0, PF.rk1, a0, a1, a2);
            draw_phi<float, false>(nullptr, gpath, lp, PF.n_paths, n + 1, PF.rk0, PF.rk1, b0, b1, b2);
            xf.step(MF, a0, a1, a2);
            bf.add(xf, a0, a1, a2);
            xf.step(MF, b0, b1, b2);
            bf.add(xf, b0, b1, b2);
            const float c0 = (a0 + b0) * kInvSqrt2, c1 = (a1 + b1) * kInvSqrt2, c2 = (a2 + b2) * kInvSqrt2;
            xc.step(MC, c0, c1, c2);
            bc.add(xc, c0, c1, c2);
        }
        block_sums_up<NT, POLY>(xf, hsF, tid, kMlCta, PF, bf, B, [&](int t, float Ht) {
            if (t > b) accF[t * kMlCta + tid] += as_f64(Ht);
        });
        block_sums_up<NT, POLY>(xc, hsC, tid, kMlCta, PC, bc, B, [&](int t, float Ht) {
            if (t > b) accC[t * kMlCta + tid] += as_f64(Ht);
        });
#pragma unroll
        for (int t = 1; t < NT; ++t)
            if (t <= B + 1) {
                hsF[t * kMlCta + tid] = xf.rem(t);
                hsC[t * kMlCta + tid] = xc.rem(t);
            }
        sample(xf, PF, accF, b + 1);
        sample(xc, PC, accC, b + 1);
    }

    // exposure differences E^f_j - E^c_j (FP64 suffix sums of each curve's cash
    // flows), the path's CVA-contribution difference, CTA partial sums.  The
    // FP64 tile spans the FP32 block-start columns of other threads, so every
    // thread must be done with them first.
    __syncthreads();
    double* e_s = reinterpret_cast<double*>(hsF);  // [B+1][kMlCta] over hsF, hsC
    double vf = 0.0, vc = 0.0, cva_d = 0.0;
    e_s[B * kMlCta + tid] = 0.0;
    for (int j = B - 1; j >= 0; --j) {
        vf += accF[(j + 1) * kMlCta + tid];
        vc += accC[(j + 1) * kMlCta + tid];
        double e = (vf > 0.0 ? vf : 0.0) - (vc > 0.0 ? vc : 0.0);
        if (!active) e = 0.0;
        e_s[j * kMlCta + tid] = e;
        cva_d = fma(PF.cvaw[j], e, cva_d);
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    const int R = B + 3;
    for (int j = warp; j <= B; j += kMlCta / 32) {
        double sum = 0.0;
#pragma unroll
        for (int q = 0; q < kMlCta / 32; ++q) sum += e_s[j * kMlCta + lane + 32 * q];
        sum = warp_sum(sum);
        if (lane == 0) partials[(size_t)blockIdx.x * R + j] = sum;
    }
    {
        const double s1 = warp_sum(cva_d), s2 = warp_sum(cva_d * cva_d);
        if (lane == 0) {
            red_s[warp] = s1;
            red_s[kMlCta / 32 + warp] = s2;
        }
    }
    __syncthreads();
    if (tid == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kMlCta / 32; ++w) {
            s1 += red_s[w];
            s2 += red_s[kMlCta / 32 + w];
        }
        partials[(size_t)blockIdx.x * R + B + 1] = s1;
        partials[(size_t)blockIdx.x * R + B + 2] = s2;
    }
}

template <int NT, bool POLY>
static cudaError_t launch_mlmc_t(const MlmcParams& Q, double* partials, cudaStream_t s)
{
    const size_t smem = mlmc_smem_bytes(Q.fine.P.n_blocks);
    auto k = mlmc_level_kernel<NT, POLY>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (Q.fine.P.n_paths + kMlCta - 1) / kMlCta;
    k<<<(unsigned)grid, kMlCta, smem, s>>>(Q, partials);
    return cudaGetLastError();
}

cudaError_t launch_mlmc_level(int nt, const MlmcParams& Q, bool poly, double* partials, cudaStream_t s)
{
    if (nt == 51) return poly ? launch_mlmc_t<51, true>(Q, partials, s) : launch_mlmc_t<51, false>(Q, partials, s);
    if (nt == 61) return poly ? launch_mlmc_t<61, true>(Q, partials, s) : launch_mlmc_t<61, false>(Q, partials, s);
    return cudaErrorInvalidValue;
}

// The predictor-corrector's coupled level kernel: the same coupling and
// partial-sum layout, each curve the predictor-corrector valuation's path
// state (PcPath, FP32 curve and pricing, FP64 discount sums).  Shared memory
// per thread: accF, accC (B+1) FP64; hsF, hsC max(NT, B+1) FP32 block-start
// curves, reused as the FP64 exposure-difference tile.
__host__ __device__ inline size_t mlmc_pc_smem_bytes(int nt, int n_blocks)
{
    const size_t rows = (size_t)n_blocks + 1;
    const size_t hs_rows = (size_t)(nt > n_blocks + 1 ? nt : n_blocks + 1);
    return 2 * rows * kMlCta * 8 + 2 * hs_rows * kMlCta * 4 + 2 * (kMlCta / 32) * 8;
}

template <int NT, bool POLY>
__global__ void __launch_bounds__(kMlCta, 4)
    mlmc_level_kernel_pc(const __grid_constant__ MlmcPcParams Q, double* __restrict__ partials)
{
    static_assert(kMlCta == kPcCta, "PcPath addresses its shared columns with kPcCta");
    const PcParams<float>& QF = Q.fine;
    const PcParams<float>& QC = Q.coarse;
    const PathParams<float>& PF = QF.P;
    const PathParams<float>& PC = QC.P;
    extern __shared__ __align__(128) unsigned char smem[];
    const int tid = threadIdx.x;
    const int B = PF.n_blocks;
    const int rows = B + 1;
    const int hs_rows = NT > B + 1 ? NT : B + 1;
    double* accF = reinterpret_cast<double*>(smem);
    double* accC = accF + (size_t)rows * kMlCta;
    float* hsF = reinterpret_cast<float*>(accC + (size_t)rows * kMlCta);
    float* hsC = hsF + (size_t)hs_rows * kMlCta;
    double* red_s = reinterpret_cast<double*>(hsC + (size_t)hs_rows * kMlCta);

    const int64_t cta_base = (int64_t)blockIdx.x * kMlCta;
    const int64_t lp = cta_base + tid;
    const bool active = lp < PF.n_paths;
    const uint64_t gpath = PF.path_offset + (uint64_t)lp;

    PcPath<NT, float, POLY> xf, xc;
    xf.reset();
    xc.reset();
    for (int i = 0; i < rows; ++i) {
        accF[i * kMlCta + tid] = 0.0;
        accC[i * kMlCta + tid] = 0.0;
    }
    for (int t = 0; t < NT; ++t) {
        hsF[t * kMlCta + tid] = 0.f;
        hsC[t * kMlCta + tid] = 0.f;
    }
    auto sample = [&](const PcPath<NT, float, POLY>& x, const PathParams<float>& P, double* acc, int i) {
        const double xv = P.psamp[i] + (double)x.value(P, i);
        const double a = P.psum[i] + acc[i * kMlCta + tid];
        const float D = exp_t<float>((float)(-a * P.dt));
        const float mm = (float)P.m;
        const float Lb = mm * expm1_t<float>((float)xv / mm);
        acc[i * kMlCta + tid] = (double)(D * ((float)P.payA[i] * Lb - (float)P.payB[i]));
    };

    const float kInvSqrt2 = 0.70710678118654752f;
    sample(xf, PF, accF, 1);
    sample(xc, PC, accC, 1);
    for (int b = 1; b < B; ++b) {
        xf.begin_block(PF, b);
        xc.begin_block(PC, b);
        for (int k = 0; k < PC.stride; ++k) {
            const int n = b * PF.stride + 2 * k;  // the fine steps n, n+1 make coarse step b*stride_c + k
            float a0, a1, a2, b0, b1, b2;
            draw_phi<float, false>(nullptr, gpath, lp, PF.n_paths, n, PF.rk0, PF.rk1, a0, a1, a2);
            draw_phi<float, false>(nullptr, gpath, lp, PF.n_paths, n + 1, PF.rk0, PF.rk1, b0, b1, b2);
            xf.step(QF, a0, a1, a2);
            xf.step(QF, b0, b1, b2);
            xc.step(QC, (a0 + b0) * kInvSqrt2, (a1 + b1) * kInvSqrt2, (a2 + b2) * kInvSqrt2);
        }
        xf.end_block(QF, b, B, hsF, accF, tid);
        xc.end_block(QC, b, B, hsC, accC, tid);
        sample(xf, PF, accF, b + 1);
        sample(xc, PC, accC, b + 1);
    }
    // the exposure-difference tile spans other threads' FP32 columns
    __syncthreads();
    double* e_s = reinterpret_cast<double*>(hsF);  // [B+1][kMlCta] over hsF, hsC
    double vf = 0.0, vc = 0.0, cva_d = 0.0;
    e_s[B * kMlCta + tid] = 0.0;
    for (int j = B - 1; j >= 0; --j) {
        vf += accF[(j + 1) * kMlCta + tid];
        vc += accC[(j + 1) * kMlCta + tid];
        double e = (vf > 0.0 ? vf : 0.0) - (vc > 0.0 ? vc : 0.0);
        if (!active) e = 0.0;
        e_s[j * kMlCta + tid] = e;
        cva_d = fma(PF.cvaw[j], e, cva_d);
    }
    __syncthreads();
    const int warp = tid >> 5, lane = tid & 31;
    const int R = B + 3;
    for (int j = warp; j <= B; j += kMlCta / 32) {
        double sum = 0.0;
#pragma unroll
        for (int q = 0; q < kMlCta / 32; ++q) sum += e_s[j * kMlCta + lane + 32 * q];
        sum = warp_sum(sum);
        if (lane == 0) partials[(size_t)blockIdx.x * R + j] = sum;
    }
    {
        const double s1 = warp_sum(cva_d), s2 = warp_sum(cva_d * cva_d);
        if (lane == 0) {
            red_s[warp] = s1;
            red_s[kMlCta / 32 + warp] = s2;
        }
    }
    __syncthreads();
    if (tid == 0) {
        double s1 = 0.0, s2 = 0.0;
        for (int w = 0; w < kMlCta / 32; ++w) {
            s1 += red_s[w];
            s2 += red_s[kMlCta / 32 + w];
        }
        partials[(size_t)blockIdx.x * R + B + 1] = s1;
        partials[(size_t)blockIdx.x * R + B + 2] = s2;
    }
}

template <int NT, bool POLY>
static cudaError_t launch_mlmc_pc_t(const MlmcPcParams& Q, double* partials, cudaStream_t s)
{
    const size_t smem = mlmc_pc_smem_bytes(NT, Q.fine.P.n_blocks);
    auto k = mlmc_level_kernel_pc<NT, POLY>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    const int64_t grid = (Q.fine.P.n_paths + kMlCta - 1) / kMlCta;
    k<<<(unsigned)grid, kMlCta, smem, s>>>(Q, partials);
    return cudaGetLastError();
}

cudaError_t launch_mlmc_level_pc(int nt, const MlmcPcParams& Q, bool poly, double* partials, cudaStream_t s)
{
    if (nt == 51) return poly ? launch_mlmc_pc_t<51, true>(Q, partials, s) : launch_mlmc_pc_t<51, false>(Q, partials, s);
    if (nt == 61) return poly ? launch_mlmc_pc_t<61, true>(Q, partials, s) : launch_mlmc_pc_t<61, false>(Q, partials, s);
    return cudaErrorInvalidValue;
}

size_t mlmc_pc_smem(int nt, int n_blocks) { return mlmc_pc_smem_bytes(nt, n_blocks); }

size_t mlmc_smem(int n_blocks) { return mlmc_smem_bytes(n_blocks); }

int mlmc_cta() { return kMlCta; }

}  // namespace hjm
