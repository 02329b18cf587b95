// hjm_device.cuh -- shared device definitions of the GB300 HJM exposure engine.
//
// Counter-based normals (Philox4x32-10 + Box-Muller, generated in registers,
// replacing the pre-generated cuRAND buffer of simulation_gpu.cu:195-216 and
// :1057-1071), the kernel parameter block, and small warp helpers.
#pragma once

#include <cmath>
#include <cstdint>
#include <cuda_runtime.h>

namespace hjm {

constexpr int kMaxTenor = 64;   // tenor-grid capacity of every parameter array
constexpr int kFactors = 3;     // PCA factors (VOL_DIM, simulation_gpu.cu:34)
constexpr int kCta = 128;       // threads per CTA of the path kernel: one path per thread

// ---------------------------------------------------------------------------
// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11), published multipliers and
// Weyl increments.  Host and device compile the same function.
// ---------------------------------------------------------------------------
__host__ __device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
#ifdef __CUDA_ARCH__
        const uint32_t lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
        const uint32_t lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
#else
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x, p1 = (uint64_t)0xCD9E8D57u * c.z;
        const uint32_t lo0 = (uint32_t)p0, hi0 = (uint32_t)(p0 >> 32);
        const uint32_t lo1 = (uint32_t)p1, hi1 = (uint32_t)(p1 >> 32);
#endif
        c = make_uint4(hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0);
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    return c;
}

#ifdef __CUDACC__
// The same generator with the ten round keys precomputed on the host (they
// depend on the seed only, so every thread shares them): the key schedule
// drops out of the per-thread work and each round is two 32x32->64
// multiplies and two three-input XORs with a constant-bank operand.
__device__ __forceinline__ uint4 philox4x32_10_rk(uint4 c, const uint32_t* rk0, const uint32_t* rk1)
{
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        c = make_uint4((uint32_t)(p1 >> 32) ^ c.y ^ rk0[r], (uint32_t)p1, (uint32_t)(p0 >> 32) ^ c.w ^ rk1[r],
                       (uint32_t)p0);
    }
    return c;
}
#endif

// Round keys of Philox4x32-10 for a seed: round r uses (k0 + r W0, k1 + r W1).
__host__ __device__ __forceinline__ void philox_round_keys(uint32_t k0, uint32_t k1, uint32_t* rk0, uint32_t* rk1)
{
    for (int r = 0; r < 10; ++r) {
        rk0[r] = k0 + (uint32_t)r * 0x9E3779B9u;
        rk1[r] = k1 + (uint32_t)r * 0xBB67AE85u;
    }
}

// Counter of the normals of (path, step): (step, stream 0, path lo, path hi).
__host__ __device__ __forceinline__ uint4 normals_counter(uint64_t path, uint32_t step)
{
    return make_uint4(step, 0u, (uint32_t)path, (uint32_t)(path >> 32));
}

#ifdef __CUDACC__
// Three N(0,1) draws for one path-step: Box-Muller on the two uniform pairs
// a = (word >> 8) * 2^-24 in [0, 1) (exact in FP32); radius sqrt(-2 ln(1 - a)),
// angle pi (2a - 1).  FP32 with the SFU: 1 - a and the angle are one FMA each
// on the integer's conversion, the logarithm is log2 times -2 ln 2, and the
// square root is t * rsqrt(t) (t >= 2^-23 or exactly 0, which the max keeps
// finite).  The normals are inputs of both precision modes (the FP64 mode
// promotes them exactly), and the oracle consumes these very values through
// hjm_dump_normals.
// The SFU's approximate log2 and reciprocal square root with subnormals
// flushed: the operands here are never subnormal (1 - a >= 2^-24, t >= 1e-30),
// so the results equal those of the non-flushing forms without their
// subnormal checks.
__device__ __forceinline__ float lg2_ftz(float x)
{
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rsqrt_ftz(float x)
{
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

__device__ __forceinline__ void normals3(uint4 w, float& z0, float& z1, float& z2)
{
    const float u0 = (float)(w.x >> 8), u1 = (float)(w.y >> 8);
    const float u2 = (float)(w.z >> 8), u3 = (float)(w.w >> 8);
    const float kM2Ln2 = -1.38629436111989061883f;          // -2 ln 2
    const float kAng = 3.74507028e-07f;                      // 2 pi 2^-24
    const float kPi = 3.14159265358979323846f;
    const float t0 = kM2Ln2 * lg2_ftz(fmaf(-0x1p-24f, u0, 1.0f));
    const float t1 = kM2Ln2 * lg2_ftz(fmaf(-0x1p-24f, u2, 1.0f));
    const float r0 = t0 * rsqrt_ftz(fmaxf(t0, 1e-30f));
    const float r1 = t1 * rsqrt_ftz(fmaxf(t1, 1e-30f));
    float s0, c0;
    __sincosf(fmaf(kAng, u1, -kPi), &s0, &c0);
    const float c1 = __cosf(fmaf(kAng, u3, -kPi));
    z0 = r0 * c0;
    z1 = r0 * s0;
    z2 = r1 * c1;
}

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
#endif

// ---------------------------------------------------------------------------
// Kernel parameter block, passed by value (constant bank): every per-tenor
// coefficient is read as an FMA operand straight from the constant bank with a
// compile-time offset once the tenor loop is unrolled.  Replaces the
// __constant__ symbols of simulation_gpu.cu:109-119 and keeps launches
// re-entrant.
//
// Curve split.  f_n = p_n + h_n, where p_n is the deterministic curve
// (p_n = spot for the first block, then p_{n+1} = A p_n + mu dt) computed on
// the host in FP64, and h_n the stochastic part,
//   h_{n+1}[t] = h_n[t] + sum_k sv[k][t] phi_{n+1,k} + c (h_n[t+1] - h_n[t]),
// with the backward difference at the last tenor (simulation_cpu.h:96-108)
// and c = dt/dtau.  Linear, so the split is exact in exact arithmetic.
// ---------------------------------------------------------------------------
template <typename T>
struct PathParams {
    T sv[kFactors][kMaxTenor];   // sqrt(dt) * sigma_k(tau_t)
    double psamp[kMaxTenor];     // p at the sampling of tenor i: p_{stride*i-1}[i]
    double psum[kMaxTenor];      // sum_{n < stride*i} p_n[i]
    double payA[kMaxTenor];      // cash flow of date i: D_i * (payA[i] * L_i - payB[i])
    double payB[kMaxTenor];
    double cvaw[kMaxTenor];      // (1-R)(exp(-l t_{j-1}) - exp(-l t_j)); cvaw[0] = 0
    T c;                         // dt / dtau
    double dt;
    double m;                    // 1 / dtau: LIBOR from the sampled forward, m (e^{f/m} - 1)
    uint32_t key0, key1;         // Philox key = seed
    uint32_t rk0[10], rk1[10];   // its round keys
    double inv_c;                // dtau / dt (FP64 block-sum recovery)
    uint64_t path_offset;        // global index of this launch's first path
    int64_t n_paths;
    int64_t ld;                  // row stride (elements) of the exposure store
    int n_blocks;                // sampled dates B = n_steps / stride
    int stride;                  // Euler steps per block (dtau / dt)
    int store_exposures;         // write per-path exposures [date][path]
    // Polynomial volatility factors, sqrt(dt) sigma_k(T) = sum_d svc[k][d] T^d
    // (degree <= 2): used by the kernels' polynomial form only.
    double svc[kFactors][3];
    double k1, k2;               // c dtau, c dtau^2
    T tau[kMaxTenor];            // tau_t = dtau t
    // Growth-scaled convection.  After n' Euler steps of the stochastic part
    // the kernels hold v = h (1 + rr)^n' instead of h, rr = c / (1 - c) rounded
    // to T once.  The upwind step h[t] + c (h[t+1] - h[t]) then reads
    //   v'[t] = v[t] + rr v[t+1]                     (t < L, one FMA),
    //   v'[L] = v[L] + rr (2 v[L] - v[L-1])          (backward difference),
    // plus the noise times (1 + rr)^(n'+1): exactly the reference scheme for
    // c_eff = rr / (1 + rr) (c to within T's rounding), with every constant
    // derived from the one rounded rr so that the homogeneous step stays
    // consistent.  v is never rescaled (its growth is at most e^(number of
    // tenors)); h = v / (1 + rr)^n' is formed only where it is read.
    T gblk[kMaxTenor];           // (1 + rr)^-(b-1) stride: the scale at the start of block b
    T igblk[kMaxTenor];          // its inverse
    T rr;                        // c / (1 - c)
    T qm;                        // 1 / (1 + rr): per-step factor of the scale
    T ip;                        // 1 + rr: per-step factor of the inverse scale
    T m2k2;                      // -2 c dtau^2: the polynomial form's last-tenor source per unit W
    double inv_m;                // dtau = 1 / m: the LIBOR's exponent x / m as a product
};

// Host: the growth-scale constants of PathParams from c = dt / dtau, k2 and
// the block layout.
template <typename T>
inline void fill_growth_scale(PathParams<T>& P, double c, double k2, int stride, int n_blocks)
{
    const T rr = (T)(c / (1.0 - c));
    const double base = 1.0 + (double)rr;  // exact in double for T = float
    for (int b = 0; b < kMaxTenor; ++b) {
        const double e = (b >= 1 && b <= n_blocks) ? (double)((b - 1) * stride) : 0.0;
        P.gblk[b] = (T)std::pow(base, -e);
        P.igblk[b] = (T)std::pow(base, e);
    }
    P.rr = rr;
    P.qm = (T)(1.0 / base);
    P.ip = (T)base;
    P.m2k2 = (T)(-2.0 * k2);
}

#ifdef __CUDACC__
// Exact FP32 -> FP64 widening with integer operations: the conversion
// instruction issues on the FP64 pipe, the bound of the FP64 path kernel, and
// these bit moves do not.  Exact for zero and normal numbers; the Box-Muller
// outputs are zero or at least ~1e-12 in magnitude, never subnormal, and a
// subnormal input would give a signed zero.
__device__ __forceinline__ double widen_f32(float f)
{
    const uint32_t u = __float_as_uint(f);
    const uint32_t mag = u & 0x7fffffffu;
    const bool normal = mag >= 0x00800000u;
    const uint32_t hi = (u & 0x80000000u) | (normal ? (mag >> 3) + 0x38000000u : 0u);
    const uint32_t lo = normal ? (mag << 29) : 0u;
    return __hiloint2double((int)hi, (int)lo);
}

// A float or double as a double, the float by widen_f32 (for the FP64 folds of
// FP32 block sums: no FP64-pipe conversion per fold)
__device__ __forceinline__ double as_f64(float f) { return widen_f32(f); }
__device__ __forceinline__ double as_f64(double d) { return d; }

// The three normals of (path, step): Philox in registers, or read from a
// caller-supplied buffer laid out [step][3][path] (coalesced across threads).
template <typename T, bool EXT>
__device__ __forceinline__ void draw_phi(const double* __restrict__ ext, uint64_t gpath, int64_t lp, int64_t n_paths,
                                         int n, const uint32_t* rk0, const uint32_t* rk1, T& phi0, T& phi1, T& phi2)
{
    if constexpr (EXT) {
        const size_t np = (size_t)n_paths;
        const size_t base = (size_t)n * 3 * np + (size_t)lp;
        phi0 = (T)__ldg(ext + base);
        phi1 = (T)__ldg(ext + base + np);
        phi2 = (T)__ldg(ext + base + 2 * np);
    } else {
        const uint4 w = philox4x32_10_rk(normals_counter(gpath, (uint32_t)n), rk0, rk1);
        float z0, z1, z2;
        normals3(w, z0, z1, z2);
        if constexpr (sizeof(T) == 8) {
            phi0 = widen_f32(z0);
            phi1 = widen_f32(z1);
            phi2 = widen_f32(z2);
        } else {
            phi0 = z0;
            phi1 = z1;
            phi2 = z2;
        }
    }
}

// Static selection of a register-array element by a runtime index (uniform
// across the warp): keeps the arrays in registers.
template <int NT, typename T>
__device__ __forceinline__ T select_reg(const T (&a)[NT], int i)
{
    T r = a[0];
#pragma unroll
    for (int t = 1; t < NT; ++t) r = (t == i) ? a[t] : r;
    return r;
}
#endif

}  // namespace hjm
