/*
 * hjm_cva.h -- C ABI of the GB300 HJM exposure / CVA engine (libhjmcva.so).
 *
 * This is the boundary that replaces the reference's GPU entry point
 * (mahsanchez/cva_hjm_cuda simulation_gpu.h:12,14 -> simulation_gpu.cu:956-1250,
 * __calculateExposureMultiGPU).  The C++ drop-in for those two overloads is
 * declared in hjm_dropin.h and is implemented on top of these functions.
 *
 * Conventions
 *   - Every function returns an hjm_status; nothing throws across the ABI.
 *     hjm_last_error(ctx) gives the message of the last failure on ctx
 *     (ctx may be NULL for failures of hjm_ctx_create).
 *   - Pointers named *_host are host memory owned by the caller.
 *   - A context owns one device, one CUDA stream and its device buffers.
 *     Calls on one context must not overlap; distinct contexts are
 *     independent and may be driven from different threads.  (The reference
 *     writes global __constant__ symbols and is not re-entrant,
 *     simulation_gpu.cu:109-119, 1032-1035.)
 *   - Arrays on the tenor grid have n_tenor entries, 2 <= n_tenor <= 64.
 *     Volatility tables are factor-major, vol[k * n_tenor + t], three factors
 *     (simulation_gpu_testing.cpp:47-63; VOL_DIM = 3 in simulation_gpu.cu:34).
 *   - Paths are numbered globally: path p uses the Philox4x32-10 counter
 *     (step, 0, p lo, p hi) under key (seed lo, seed hi), so a run over paths
 *     [path_offset, path_offset + n_paths) draws exactly the normals those
 *     paths draw in any larger run.
 */
#ifndef HJM_CVA_H
#define HJM_CVA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HJM_MAX_TENOR 64
#define HJM_N_FACTOR 3
#define HJM_N_VOL_COEF 9 /* three factors x polynomial degree <= 2 */

typedef struct hjm_ctx hjm_ctx;

typedef enum hjm_status {
    HJM_OK = 0,
    HJM_ERR_INVALID_ARGUMENT = 1,
    HJM_ERR_UNSUPPORTED = 2,
    HJM_ERR_CUDA = 3,
    HJM_ERR_OUT_OF_MEMORY = 4,
    HJM_ERR_NOT_CONFIGURED = 5,
    HJM_ERR_NO_DEVICE = 6
} hjm_status;

typedef enum hjm_precision {
    /* curve evolution, swap pricing and reductions in FP64 */
    HJM_PRECISION_FP64 = 0,
    /* curve evolution and swap pricing in FP32; the deterministic drift
     * integral, the discount accumulation and the EE/CVA reductions in FP64 */
    HJM_PRECISION_MIXED = 1
} hjm_precision;

/* Output layout of hjm_run / hjm_run_with_normals: cva_out[0..3] */
#define HJM_CVA_VALUE 0
#define HJM_CVA_STDERR 1    /* Monte Carlo standard error of the CVA estimate */
#define HJM_CVA_DHAZARD 2   /* dCVA / d(hazard rate), exact from EE */
#define HJM_CVA_OUT_LEN 3

/* ---- library / context --------------------------------------------------- */
const char* hjm_version(void);
/* Message of the last failure on ctx (or of the calling thread when ctx is NULL). */
const char* hjm_last_error(const hjm_ctx* ctx);

/* Create a context on CUDA device `device`.  Replaces the per-GPU set-up of
 * simulation_gpu.cu:989-1043 (allocation, generator, constant uploads). */
hjm_status hjm_ctx_create(int device, hjm_ctx** out);
hjm_status hjm_ctx_destroy(hjm_ctx* ctx);
/* Launch on a caller-owned cudaStream_t instead of the context's own stream
 * (NULL restores the context's stream). */
hjm_status hjm_ctx_set_stream(hjm_ctx* ctx, void* cuda_stream);

/* Cap on the device memory the context's buffers may hold, in bytes (0, the
 * default: no cap).  A call whose buffers would grow past it fails with
 * HJM_ERR_OUT_OF_MEMORY before anything is allocated or freed, exactly as a
 * failed cudaMalloc is reported; the context stays usable (a later call that
 * fits, or one after the cap is raised, runs normally).  Buffers already held
 * are kept when the cap is lowered.  hjm_ctx_memory_in_use reports the bytes
 * held now. */
hjm_status hjm_ctx_set_memory_limit(hjm_ctx* ctx, int64_t bytes);
hjm_status hjm_ctx_memory_in_use(hjm_ctx* ctx, int64_t* bytes);

/* Keep the per-path exposures of every valuation on the device (for
 * hjm_get_exposures); they are always kept when a PFE is requested. */
hjm_status hjm_ctx_keep_exposures(hjm_ctx* ctx, int32_t keep);

/* Time scheme of the Musiela SDE.  HJM_SCHEME_EULER (default) is the
 * reference's Euler step (simulation_cpu.h:37-54); HJM_SCHEME_PREDICTOR_CORRECTOR
 * (the reference's doc/TODO:3) averages the drift term mu + dF/dtau at the
 * curve and at its Euler prediction: f' = f + (a(f) + a(f*)) dt / 2 + xi.
 * Valuations (both precisions, the table and the decomposed volatility step),
 * hjm_run_adjoint (with checkpoint_every = 0 for the predictor-corrector) and
 * hjm_run_mlmc support both; hjm_run_static the Euler step only. */
#define HJM_SCHEME_EULER 0
#define HJM_SCHEME_PREDICTOR_CORRECTOR 1
hjm_status hjm_ctx_set_scheme(hjm_ctx* ctx, int32_t scheme);

/* Polynomial volatility decomposition.  When every volatility factor is a
 * polynomial of degree <= 2 in the tenor T (given by hjm_set_market_poly, or a
 * table that hjm_set_market finds to be one to 1e-12 of each row's scale, as
 * the configured workloads' synthetic factors are), the kernels
 * carry the stochastic curve as S + U T + W T^2 plus a remainder driven only at
 * the last tenor, instead of adding the three factor columns to every tenor
 * each step (simulation_gpu.cu:153-180).  enable = 0 forces the generic
 * table-driven step; default 1.  A table that is no quadratic but a cubic in
 * each factor up to a residual of at most 2^-20 of the factor's scale (a PCA
 * table printed to a fixed number of decimals, as the reference's own
 * simulation_gpu_testing.cpp:47-63, whose factors 2 and 3 are cubics to
 * 1.1e-7) runs, in Euler valuations, the cubic decomposition: in FP64 with
 * the residual's impulse responses carried beside the remainder's, in mixed
 * precision without the residual (below FP32's resolution of the loadings);
 * the predictor-corrector scheme, the adjoint and MLMC run the table step on
 * it.
 * hjm_ctx_vol_decomposition reports what the current market runs: 0 the
 * table step, 1 the decomposition, 2 the decomposition with factor k of
 * degree <= k (three zero coefficients), 3 the cubic decomposition with a
 * residual table. */
hjm_status hjm_ctx_set_vol_decomposition(hjm_ctx* ctx, int32_t enable);
hjm_status hjm_ctx_vol_decomposition(hjm_ctx* ctx, int32_t* active);

/* Transport form of the remainder.  The pricing reads the stochastic curve only at each
 * date's own tenor.  With the polynomial decomposition the remainder, driven
 * only at the last tenor (the last two for the predictor-corrector), is either
 * convected over the live tenors every step (HJM_REMAINDER_CONVECT) or carried,
 * for each date still to be sampled, as its value and running sum in impulse
 * responses of the convection (HJM_REMAINDER_RESPONSE: one double-FP32 term
 * per such date per step, on the FP32 pipe; the remainder is ~1e-5 of the
 * curve; the polynomial parts S, U, W then advance as double-FP32 sums in a
 * moving frame, with FP64 only at the sampled dates).  With a volatility
 * table of any shape (no decomposition) the whole stochastic curve is either
 * convected with the noise injected at every tenor (four FP64 FMAs per live
 * tenor per step), or carried in the response form as double-FP32 sums of
 * the three factors' impulse responses (three terms per date per step).
 * Every response form takes any number of dates: a run with more than
 * HJM_RESPONSE_MAX_DATES is priced in windows of at most that many dates, one
 * launch each, the later windows passing each path's later cash flows to the
 * earlier ones.  HJM_REMAINDER_AUTO (default) takes the response form for
 * every FP64 valuation.  Both time schemes; the forms agree to rounding
 * (per-path exposures within ~1e-13 of the exposure scale).  Mixed precision
 * with the decomposition carries the remainder as FP32
 * impulse-response sums (one packed FMA per date per step) when the dates
 * whose responses ever reach 2^-30 of the source fit 16 slots (the 10y swap's
 * 20 dates on 51 tenors: 8), else convects it in FP32 pairs (the 25y swap,
 * the 30y netting set); the two agree to FP32 rounding (~1e-7 of the
 * exposure scale).  AUTO and RESPONSE take it where it fits, under either
 * scheme (the predictor-corrector's only when its last date does not sample
 * the last tenor), and in hjm_run_adjoint without checkpoints (Euler); the
 * adjoint with checkpoints, the predictor-corrector's adjoint and MLMC's
 * coupled levels convect.  The report names the form a valuation ran
 * ("remainder"). */
#define HJM_REMAINDER_AUTO 0
#define HJM_REMAINDER_CONVECT 1
#define HJM_REMAINDER_RESPONSE 2
#define HJM_RESPONSE_MAX_DATES 24
hjm_status hjm_ctx_set_remainder_form(hjm_ctx* ctx, int32_t form);
/* The transport form of the last valuation enqueued: HJM_REMAINDER_CONVECT or
 * HJM_REMAINDER_RESPONSE. */
hjm_status hjm_ctx_remainder_form(hjm_ctx* ctx, int32_t* form);

/* ---- inputs --------------------------------------------------------------- */
/* Market: spot forward curve, volatility factors, and the drift.  With
 * drift_host == NULL the Musiela no-arbitrage drift is computed in FP64 by the
 * trapezoid rule on the tenor grid.  Replaces the cudaMemcpyToSymbol uploads of
 * simulation_gpu.cu:1032-1035 (spot, drift, volatilities). */
hjm_status hjm_set_market(hjm_ctx* ctx, int32_t n_tenor, double dtau, const double* spot_host,
                          const double* vol_host, int32_t n_factor, const double* drift_host);

/* One interest-rate swap (product.h:4-18 InterestRateSwap: notional, K, and
 * the accrual table of simulation_gpu.cu:1032).  payer != 0 pays fixed:
 * cash flow D * N * alpha * (L - K); a receiver swap has the opposite sign. */
hjm_status hjm_set_swap(hjm_ctx* ctx, double notional, double fixed_rate, const double* accrual_host,
                        int32_t payer);

/* A netting set of n_swaps swaps on the tenor grid, netted before max(., 0).
 * Swap s accrues dtau on periods 1..n_periods[s].  Generalises the single
 * swap of simulation_cpu.h:269-296. */
hjm_status hjm_set_netting_set(hjm_ctx* ctx, int32_t n_swaps, const double* notional_host,
                               const double* fixed_rate_host, const int32_t* n_periods_host,
                               const int32_t* payer_host);

/* ---- forward valuation ---------------------------------------------------- */
/* Simulate n_paths paths of n_steps Euler steps of size dt (n_steps must be a
 * multiple of stride = dtau / dt; the reference's block loop,
 * simulation_cpu.h:413, simulation_gpu.cu:594-669), price the product at the
 * end of every block, and reduce.
 *   ee_out      [n_tenor]  expected exposure EE(t_j), t_j = j * dtau (zero
 *                          beyond the last sampled date) -- the reference's
 *                          expected_exposure output (simulation_gpu.cu:1177-1179)
 *   pfe_out     [n_tenor]  PFE(t_j) at pfe_quantile (may be NULL; then
 *                          pfe_quantile is ignored)
 *   cva_out     [HJM_CVA_OUT_LEN]  CVA, its MC standard error, dCVA/dhazard,
 *               CVA = (1-R) sum_j EE(t_j) (exp(-l t_{j-1}) - exp(-l t_j)).
 * Host buffers; blocks until the results are on the host. */
hjm_status hjm_run(hjm_ctx* ctx, int64_t n_paths, int32_t n_steps, double dt, uint64_t seed,
                   uint64_t path_offset, int32_t precision, double hazard_rate, double recovery,
                   double pfe_quantile, double* ee_out, double* pfe_out, double* cva_out);

/* The same valuation, enqueued on the context's stream without any host copy
 * or synchronisation; results stay on the device until hjm_fetch_results. */
hjm_status hjm_enqueue(hjm_ctx* ctx, int64_t n_paths, int32_t n_steps, double dt, uint64_t seed,
                       uint64_t path_offset, int32_t precision, double hazard_rate, double recovery,
                       double pfe_quantile);
hjm_status hjm_fetch_results(hjm_ctx* ctx, double* ee_out, double* pfe_out, double* cva_out);

/* The valuation on caller-supplied normals, normals_host[path][step][3]
 * (the reference's layout, simulation_cpu.h:205-207, simulation_gpu.cu:410).
 * Used to feed the reference's own draws to the kernels. */
hjm_status hjm_run_with_normals(hjm_ctx* ctx, int64_t n_paths, int32_t n_steps, double dt,
                                const double* normals_host, int32_t precision, double hazard_rate,
                                double recovery, double pfe_quantile, double* ee_out,
                                double* pfe_out, double* cva_out);

/* Exposures of the last valuation, date-major: out[j * n_paths + p] for
 * j = 0 .. n_dates-1 with n_dates = n_steps / stride + 1 (the exposure
 * matrix of simulation_gpu.cu:1003 / simulation_cpu.h:362, transposed). */
hjm_status hjm_get_exposures(hjm_ctx* ctx, double* out_host, int64_t capacity);

/* Exposures of the paths [path_begin, path_begin + n) of the last valuation,
 * date-major as hjm_get_exposures: out[j * n + p] for path path_begin + p.
 * Copies only that slice (one strided device-to-host copy; the FP32 store of
 * a mixed-precision run is widened on the host), so a caller can inspect a
 * few paths of a run whose whole store would not fit in host memory.  No
 * counterpart in the reference, which returns the expected exposure only. */
hjm_status hjm_get_exposure_paths(hjm_ctx* ctx, int64_t path_begin, int64_t n, double* out_host);

/* ---- multi-level Monte Carlo --------------------------------------------------- */
/* EE and CVA by multi-level Monte Carlo (the reference's doc/TODO:15): level l
 * runs the context's time scheme with dt / 2^l and n_steps 2^l; level 0 is the plain
 * mixed-precision valuation on n_paths[0] paths, level l >= 1 estimates
 * E[P_l - P_{l-1}] on n_paths[l] paths whose fine and coarse curves share the
 * Brownian increments (coarse normal = (phi_a + phi_b) / sqrt 2).  The outputs
 * sum the levels: ee_out [n_tenor], cva_out [HJM_CVA_OUT_LEN] (the standard
 * error combines the levels' independent errors); level_out [n_levels][4] =
 * {CVA difference of the level, its standard error, device ms, paths}, the
 * inputs of the usual path allocation N_l ~ sqrt(V_l / C_l).  Mixed
 * precision, Euler or predictor-corrector; normals of level l come from path
 * index + l 2^40. */
#define HJM_MLMC_MAX_LEVELS 6
hjm_status hjm_run_mlmc(hjm_ctx* ctx, int32_t n_levels, const int64_t* n_paths, int32_t n_steps, double dt,
                        uint64_t seed, double hazard_rate, double recovery, double* ee_out, double* cva_out,
                        double* level_out);

/* ---- report ----------------------------------------------------------------- */
/* The results of the last valuation fetched (hjm_run, hjm_fetch_results,
 * hjm_run_with_normals), of the last hjm_run_adjoint or of the last
 * hjm_run_mlmc (kind "mlmc", with its levels), with the run's inputs,
 * written to a file: JSON (one object: run, cva, cva_stderr, dcva_dhazard,
 * dates, ee and pfe, or the sensitivities) or CSV (key,value lines, then one
 * row per tenor).  Numbers round-trip (17 significant digits).  The reference
 * prints its 51 EE values on stdout (simulation_gpu_testing.cpp:248-252). */
#define HJM_REPORT_JSON 0
#define HJM_REPORT_CSV 1
hjm_status hjm_write_report(hjm_ctx* ctx, const char* path, int32_t format);

/* ---- market input step ------------------------------------------------------ */
/* Volatility factors from historical forward curves (the step before the path:
 * the reference hard-codes its result, simulation_gpu_testing.cpp:47-63, and
 * lists the calibration as a to-do, doc/TODO:13).  Principal components of the
 * covariance of the curve changes, annualised by obs_per_year (252 for daily
 * curves):
 *   curves      [n_obs][n_tenor], tenor t at T = dtau t
 *   vol_out     [n_factor][n_tenor] sqrt(lambda_k) e_k (factor-major, the
 *               layout hjm_set_market takes); the component of largest
 *               magnitude of each factor is positive
 *   eigval_out  [n_factor] lambda_k, descending (may be NULL)
 *   coef_out    [n_factor * 3] least-squares fit of factor k by a polynomial of
 *               degree min(k, 2) in T (coefficients of 1, T, T^2; the input of
 *               hjm_set_market_poly; may be NULL)
 *   explained_out  share of the total variance the factors carry (may be NULL)
 * n_factor must be 3.  Host computation in FP64; needs no GPU. */
hjm_status hjm_calibrate_pca(const double* curves, int32_t n_obs, int32_t n_tenor, double dtau,
                             double obs_per_year, int32_t n_factor, double* vol_out, double* eigval_out,
                             double* coef_out, double* explained_out);

/* ---- sensitivities ---------------------------------------------------------- */
/* Pathwise adjoint of the CVA: dCVA/d(initial forwards) [n_tenor],
 * dCVA/d(drift table) [n_tenor], dCVA/d(polynomial volatility coefficients)
 * [HJM_N_VOL_COEF] (diffusion and trapezoid-drift paths; coefficient (k,d)
 * multiplies T^d in factor k), and dCVA/d(hazard).  Curve states are
 * checkpointed every checkpoint_every steps (0 = none: the sampled states are
 * kept instead) and each date's state is recomputed from the last checkpoint
 * before it for the reverse sweep; the predictor-corrector scheme keeps the
 * sampled states (checkpoint_every must be 0).  With checkpoint_every = 0,
 * quadratic factors and the Euler step, the adjoint runs in the response
 * form where the mixed valuation does (the remainder's FP32 responses in the
 * forward pass; in the reverse sweep the remainder's adjoint at the last
 * tenor from the same table and the sampled dates' seeds): it needs no
 * forward state but the sampled one, so there is nothing to checkpoint
 * (8.3 ms at 1,048,576 paths on the 10y swap, against 16.3 ms with
 * checkpoints every 32 steps); HJM_REMAINDER_CONVECT keeps the convected
 * adjoint.  The coefficient sensitivities require a market set through
 * hjm_set_market_poly. */
hjm_status hjm_set_market_poly(hjm_ctx* ctx, int32_t n_tenor, double dtau, const double* spot_host,
                               const double* vol_coef_host /* [3][3] */);
hjm_status hjm_run_adjoint(hjm_ctx* ctx, int64_t n_paths, int32_t n_steps, double dt, uint64_t seed,
                           uint64_t path_offset, double hazard_rate, double recovery,
                           int32_t checkpoint_every, double* cva_out, double* dcva_dspot_out,
                           double* dcva_ddrift_out, double* dcva_dvolcoef_out);

/* ---- allocation-free valuation ------------------------------------------------ */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory after start-up -- a host whose pool allocator owns the whole GPU, a
 * plugin loaded into such a process, a latency-bound loop that cannot take
 * the device-wide synchronisation a cudaMalloc/cudaFree may cause.  No
 * context: all inputs are host arrays (as for hjm_set_market / hjm_set_swap /
 * hjm_run), the work is enqueued on cuda_stream (NULL = the legacy default
 * stream) and the call is synchronous: it waits for cuda_stream and returns
 * when ee_out [n_tenor] and cva_out [HJM_CVA_OUT_LEN] hold the results.  Its
 * device memory is two fixed static arrays that each GPU loading the library
 * keeps until exit: 8.4 MB of scratch and 4 MB for a response form's table
 * (FP64, or mixed precision's), about 12.4 MB in all; it calls no cudaMalloc, cudaFree or allocating
 * library routine.  Limits: at most
 * HJM_STATIC_MAX_PATHS paths per call (larger runs fail with
 * HJM_ERR_INVALID_ARGUMENT), EE and CVA only (no PFE).  The first call on a
 * device looks up the scratch address (cudaGetSymbolAddress): make that first
 * call before any stream capture.  All calls share the scratch, so calls that
 * overlap on the GPU race; serialise them.  Errors: hjm_last_error(NULL). */
#define HJM_STATIC_MAX_PATHS 1048576
hjm_status hjm_run_static(void* cuda_stream, int32_t n_tenor, double dtau, const double* spot_host,
                          const double* vol_host, const double* drift_host, double notional, double fixed_rate,
                          const double* accrual_host, int32_t payer, int64_t n_paths, int32_t n_steps, double dt,
                          uint64_t seed, uint64_t path_offset, int32_t precision, double hazard_rate,
                          double recovery, double* ee_out, double* cva_out);

/* ---- diagnostics ------------------------------------------------------------- */
/* The device's normals for paths [path_offset, path_offset+n_paths) and steps
 * [0, n_steps): out[path][step][3], exactly the values the path kernel uses. */
hjm_status hjm_dump_normals(hjm_ctx* ctx, int64_t n_paths, uint64_t path_offset, int32_t n_steps,
                            uint64_t seed, double* out_host);
/* Raw Philox4x32-10 words for counter (step, 0, p lo, p hi), key = seed:
 * out[p * 4 + i]. */
hjm_status hjm_philox_words(hjm_ctx* ctx, int64_t n_paths, uint64_t path_offset, uint32_t step,
                            uint64_t seed, uint32_t* out_host);
/* Device times of the last valuation (ms): [0] path kernel, [1] reductions,
 * [2] PFE selection, [3] whole enqueue. */
hjm_status hjm_last_timings(hjm_ctx* ctx, double* ms_out /* [4] */);
/* The same four device times for each of the last n valuations (n <= 64),
 * oldest first: ms_out[4 * i + k]. */
hjm_status hjm_timing_history(hjm_ctx* ctx, int32_t n, double* ms_out /* [4 * n] */);
/* Counters of the last valuation: [0] kernels launched, [1] bytes copied
 * host -> device (kernel parameter blocks and caller arrays), [2] bytes copied
 * device -> host (results). */
hjm_status hjm_last_stats(hjm_ctx* ctx, int64_t* stats_out /* [3] */);
/* Sustained FMA throughput of this device in TFLOP/s (2 flops per FMA) for
 * precision HJM_PRECISION_FP64 (DFMA) or HJM_PRECISION_MIXED (FFMA). */
hjm_status hjm_measure_fma_peak(hjm_ctx* ctx, int32_t precision, double* tflops_out);

#ifdef __cplusplus
}
#endif
#endif /* HJM_CVA_H */
