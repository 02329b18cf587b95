/*
 * hjm_oracle.c -- TEST INFRASTRUCTURE ONLY (the oracle).
 *
 * A plain-C CPU restatement of the reference's Monte Carlo HJM exposure path
 * (mahsanchez/cva_hjm_cuda, simulation_cpu.h).  Only tests/, the smoke check
 * and bench.py's CPU-baseline leg may load this file's library; the product
 * (cva_hjm_cuda_gb300/) never links, imports or falls back to it.
 *
 * What is restated, with the reference lines each part follows:
 *   - Musiela SDE step            simulation_cpu.h:37-54   (__musiela_sde)
 *   - forward difference dF       simulation_cpu.h:96-108  (dFau)
 *   - one 0.5y block of a path    simulation_cpu.h:188-262 (__generatePaths_kernel_cpu)
 *   - driver loop over blocks     simulation_cpu.h:405-436 (calculateExposureCPU)
 *   - swap MtM / exposure         simulation_cpu.h:269-296 (__calculateExposure_kernel)
 *   - expected exposure (mean)    simulation_cpu.h:301-343 (blas_gemv + copy-out)
 * Arithmetic is written in the reference's operation order and built with
 * -ffp-contract=off so that it reproduces the reference bit for bit on the
 * same normals (checked against the reference compiled from its own sources
 * and against golden vectors made from it).
 *
 * Deliberate differences from a literal copy, all of which the reference's
 * own driver configuration makes irrelevant (dt = 0.01, dtau = 0.5):
 *   - the SDE uses the caller's dt and dtau; the reference's CPU path always
 *     uses its default arguments 0.01 / 0.5 (simulation_cpu.h:419-431);
 *   - numeraires that no block writes are zero, so their cash flows are
 *     zero; the reference leaves them uninitialised (simulation_cpu.h:358-359);
 *   - the exposure loop stops at the last tenor; the reference also writes
 *     exposure[51], one past the row (simulation_cpu.h:288);
 *   - the tenor count is an argument; the reference fixes it at 51.
 *
 * Not in the reference at all (new, parity unpinned by it): the trapezoid
 * no-arbitrage drift, CVA, PFE quantiles, per-path CVA contributions, the
 * Philox4x32-10 normal generator and the multi-threaded timing driver.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORACLE_MAX_TENOR 128
#define ORACLE_N_FACTOR 3

/* ------------------------------------------------------------------------ */
/* Philox4x32-10: Salmon, Moraes, Dror, Shaw, "Parallel Random Numbers: As  */
/* Easy as 1, 2, 3", SC'11.  Multipliers and Weyl key increments are the   */
/* published ones.                                                           */
/* ------------------------------------------------------------------------ */
void oracle_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4])
{
    uint32_t x0 = ctr[0], x1 = ctr[1], x2 = ctr[2], x3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)0xD2511F53u * (uint64_t)x0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * (uint64_t)x2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        x0 = hi1 ^ x1 ^ k0;
        x1 = lo1;
        x2 = hi0 ^ x3 ^ k1;
        x3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

/* Normals for (path, step): counter = (step, stream 0, path lo, path hi),
 * key = seed; Box-Muller on the two uniform pairs a = (word >> 8) * 2^-24,
 * radius sqrt(-2 log(1 - a0)), angle pi * (2 a1 - 1); first three values used.
 * The host's logf/sinf/cosf differ from the device's in the last bits, so
 * these are for CPU-only runs; parity tests feed device-dumped normals. */
static float top24(uint32_t x) { return (float)(x >> 8) * 5.9604644775390625e-08f; }

static void normals3(uint64_t seed, uint64_t path, uint32_t step, double phi[3])
{
    uint32_t ctr[4] = {step, 0u, (uint32_t)path, (uint32_t)(path >> 32)};
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    uint32_t o[4];
    oracle_philox4x32_10(ctr, key, o);
    const float pi = 3.14159265358979323846f;
    float r0 = sqrtf(-2.0f * logf(1.0f - top24(o[0])));
    float a0 = pi * (2.0f * top24(o[1]) - 1.0f);
    float r1 = sqrtf(-2.0f * logf(1.0f - top24(o[2])));
    float a1 = pi * (2.0f * top24(o[3]) - 1.0f);
    phi[0] = (double)(r0 * cosf(a0));
    phi[1] = (double)(r0 * sinf(a0));
    phi[2] = (double)(r1 * cosf(a1));
}

void oracle_normals_host(uint64_t seed, uint64_t path0, int n_paths, int n_steps, double* out)
{
    for (int p = 0; p < n_paths; ++p)
        for (int n = 0; n < n_steps; ++n)
            normals3(seed, path0 + (uint64_t)p, (uint32_t)n, out + ((size_t)p * n_steps + n) * 3);
}

/* ------------------------------------------------------------------------ */
/* Reference restatement                                                     */
/* ------------------------------------------------------------------------ */

/* simulation_cpu.h:37-54.  The reference ignores its sqrt_dt argument and
 * recomputes sqrt(dt) (line 43); so does this. */
static double musiela_sde(double drift, double vol0, double vol1, double vol2,
                          double phi0, double phi1, double phi2,
                          double dF, double rate0, double dtau, double dt)
{
    double vol_sum = vol0 * phi0;
    vol_sum += vol1 * phi1;
    vol_sum += vol2 * phi2;
    vol_sum *= sqrt(dt);
    double dfbar = drift * dt;
    dfbar += vol_sum;
    dfbar += (dF / dtau) * dt;
    return rate0 + dfbar;
}

/* simulation_cpu.h:96-108: forward difference, backward at the last tenor. */
static double dfau(int t, int nt, const double* rates)
{
    return (t == nt - 1) ? rates[t] - rates[t - 1] : rates[t + 1] - rates[t];
}

typedef struct {
    int nt, stride, n_steps;
    double dtau, dt;
    const double *spot, *vol, *drift, *accrual;
    double notional, strike, sign;
    /* netting set (new, not in the reference): cash flow of date i is
     * D_i * (payA[i] * L_i - payB[i]), payA = sum of signed notional x accrual,
     * payB = the same times each swap's fixed rate; NULL = the single swap */
    const double *payA, *payB;
    /* time scheme (new, not in the reference; its doc/TODO:3 lists it):
     * 0 = the reference's Euler step, 1 = predictor-corrector (Heun) on the
     * drift term a(f) = mu + dF/dtau: f* = Euler step, then
     * f' = f + (a(f) + a(f*)) dt / 2 + sqrt(dt) sum_k sigma_k phi_k */
    int scheme;
} oracle_model;

/* One path: simulation_cpu.h:188-262 called from the block loop at :413-436,
 * then the exposure of :269-296.  numer_x/numer_y are zeroed first. */
static void simulate_path(const oracle_model* M, const double* normals_path,
                          double* exposure /* [nt] */, double* cash_flows /* [nt] */)
{
    const int nt = M->nt;
    double f[ORACLE_MAX_TENOR], f0[ORACLE_MAX_TENOR], acc[ORACLE_MAX_TENOR];
    double numer_x[ORACLE_MAX_TENOR], numer_y[ORACLE_MAX_TENOR];
    memset(f, 0, sizeof(f));
    memset(f0, 0, sizeof(f0));
    memset(acc, 0, sizeof(acc));
    memset(numer_x, 0, sizeof(numer_x));
    memset(numer_y, 0, sizeof(numer_y));

    for (int path = 0; path < M->n_steps; path += M->stride) {      /* :413 */
        for (int s = 0; s < M->stride; ++s) {                        /* :203 */
            const double* phi = normals_path + (size_t)(path + s) * 3; /* :205-207 */
            double fs[ORACLE_MAX_TENOR];
            if (path != 0 && M->scheme == 1)                         /* predictor: the Euler step */
                for (int t = 0; t < nt; ++t)
                    fs[t] = musiela_sde(M->drift[t], M->vol[t], M->vol[nt + t], M->vol[2 * nt + t],
                                        phi[0], phi[1], phi[2], dfau(t, nt, f), f[t], M->dtau, M->dt);
            for (int t = 0; t < nt; ++t) {                           /* :210 */
                double rate;
                if (path == 0) {
                    rate = M->spot[t];                               /* :212-213 */
                } else if (M->scheme == 1) {
                    /* corrector: the average of the drift terms at f and f* */
                    const double a0 = M->drift[t] + dfau(t, nt, f) / M->dtau;
                    const double a1 = M->drift[t] + dfau(t, nt, fs) / M->dtau;
                    double vol_sum = M->vol[t] * phi[0];
                    vol_sum += M->vol[nt + t] * phi[1];
                    vol_sum += M->vol[2 * nt + t] * phi[2];
                    rate = f[t] + 0.5 * (a0 + a1) * M->dt + vol_sum * sqrt(M->dt);
                } else {
                    double dF = dfau(t, nt, f);
                    rate = musiela_sde(M->drift[t], M->vol[t], M->vol[nt + t], M->vol[2 * nt + t],
                                       phi[0], phi[1], phi[2], dF, f[t], M->dtau, M->dt);
                }
                acc[t] += rate;                                      /* :235 */
                f0[t] = rate;                                        /* :238 */
            }
            for (int t = 0; t < nt; ++t) f[t] = f0[t];              /* :242-244 */
        }
        int lindex = (path + M->stride) / M->stride;                 /* :248 */
        if (lindex < nt) {
            numer_x[lindex] = f0[lindex];                            /* :249 */
            numer_y[lindex] = exp(-acc[lindex] * M->dt);             /* :250 */
        }
    }

    /* :269-296 */
    double m = 1.0 / M->dtau;
    for (int t = 0; t < nt; ++t) {
        double forward_rate = numer_x[t];
        double discount_factor = numer_y[t];
        double libor = m * (exp(forward_rate / m) - 1.0);
        if (M->payA)
            cash_flows[t] = discount_factor * (M->payA[t] * libor - M->payB[t]);
        else
            cash_flows[t] = discount_factor * M->notional * M->accrual[t] * ((libor - M->strike) * M->sign);
    }
    for (int t = 0; t < nt; ++t) {
        double sum = 0.0;
        for (int i = t + 1; i < nt; ++i) sum += cash_flows[i];
        exposure[t] = (sum > 0.0) ? sum : 0.0;
    }
}

static int model_init(oracle_model* M, int n_tenor, double dtau, double dt, int n_steps,
                      const double* spot, const double* vol, const double* drift,
                      const double* accrual, double notional, double strike, double sign)
{
    if (n_tenor < 2 || n_tenor > ORACLE_MAX_TENOR || dt <= 0.0 || dtau <= 0.0 || n_steps <= 0) return -1;
    M->stride = (int)(dtau / dt + 0.5);
    if (M->stride <= 0 || n_steps % M->stride != 0) return -2;
    if (n_steps / M->stride > n_tenor - 1) return -3;
    M->nt = n_tenor; M->dtau = dtau; M->dt = dt; M->n_steps = n_steps;
    M->spot = spot; M->vol = vol; M->drift = drift; M->accrual = accrual;
    M->notional = notional; M->strike = strike; M->sign = sign;
    M->payA = NULL; M->payB = NULL;
    M->scheme = 0;
    return 0;
}

/* Per-path exposures for given normals ([path][step][3], the reference's
 * layout, simulation_cpu.h:424).  exposures is [n_paths][n_tenor]. */
int oracle_exposure_paths(int n_tenor, double dtau, double dt, int n_steps,
                          const double* spot, const double* vol, const double* drift,
                          const double* accrual, double notional, double strike, double sign,
                          int n_paths, const double* normals, double* exposures)
{
    oracle_model M;
    int rc = model_init(&M, n_tenor, dtau, dt, n_steps, spot, vol, drift, accrual, notional, strike, sign);
    if (rc) return rc;
    double cf[ORACLE_MAX_TENOR];
    for (int p = 0; p < n_paths; ++p)
        simulate_path(&M, normals + (size_t)p * n_steps * 3, exposures + (size_t)p * n_tenor, cf);
    return 0;
}

/* The same with a time scheme: 0 = Euler (the reference), 1 = predictor-corrector. */
int oracle_exposure_paths_scheme(int scheme, int n_tenor, double dtau, double dt, int n_steps,
                                 const double* spot, const double* vol, const double* drift,
                                 const double* accrual, double notional, double strike, double sign,
                                 int n_paths, const double* normals, double* exposures)
{
    oracle_model M;
    int rc = model_init(&M, n_tenor, dtau, dt, n_steps, spot, vol, drift, accrual, notional, strike, sign);
    if (rc) return rc;
    if (scheme != 0 && scheme != 1) return -4;
    M.scheme = scheme;
    double cf[ORACLE_MAX_TENOR];
    for (int p = 0; p < n_paths; ++p)
        simulate_path(&M, normals + (size_t)p * n_steps * 3, exposures + (size_t)p * n_tenor, cf);
    return 0;
}

/* The same valuation for a netting set given by its per-date payoff vectors. */
int oracle_exposure_paths_netting(int n_tenor, double dtau, double dt, int n_steps,
                                  const double* spot, const double* vol, const double* drift,
                                  const double* payA, const double* payB,
                                  int n_paths, const double* normals, double* exposures)
{
    oracle_model M;
    int rc = model_init(&M, n_tenor, dtau, dt, n_steps, spot, vol, drift, payA, 0.0, 0.0, 1.0);
    if (rc) return rc;
    M.payA = payA;
    M.payB = payB;
    double cf[ORACLE_MAX_TENOR];
    for (int p = 0; p < n_paths; ++p)
        simulate_path(&M, normals + (size_t)p * n_steps * 3, exposures + (size_t)p * n_tenor, cf);
    return 0;
}

/* simulation_cpu.h:301-343: EE = (1/N) * X^T * 1 (row-major gemv, beta 0). */
void oracle_expected_exposure(const double* exposures, int n_paths, int n_tenor, double* ee)
{
    const double alpha = 1.0 / (double)n_paths;
    for (int t = 0; t < n_tenor; ++t) {
        double s = 0.0;
        for (int p = 0; p < n_paths; ++p) s += exposures[(size_t)p * n_tenor + t] * 1.0;
        ee[t] = alpha * s;
    }
}

/* ------------------------------------------------------------------------ */
/* New: drift, CVA, PFE (absent from the reference)                           */
/* ------------------------------------------------------------------------ */

/* Musiela no-arbitrage drift by the trapezoid rule on the tenor grid:
 * mu_i = sum_k sigma_k(tau_i) * sum_{j=1..i} (sigma_k(tau_j)+sigma_k(tau_{j-1}))/2 * dtau. */
void oracle_trapezoid_drift(const double* vol, int n_factor, int n_tenor, double dtau, double* drift)
{
    for (int i = 0; i < n_tenor; ++i) drift[i] = 0.0;
    for (int k = 0; k < n_factor; ++k) {
        const double* s = vol + (size_t)k * n_tenor;
        double integral = 0.0;
        for (int i = 0; i < n_tenor; ++i) {
            if (i > 0) integral += 0.5 * (s[i] + s[i - 1]) * dtau;
            drift[i] += s[i] * integral;
        }
    }
}

/* CVA = (1-R) * sum_{j=1..n_dates-1} EE(t_j) * (exp(-l t_{j-1}) - exp(-l t_j)), t_j = j*dtau.
 * Also returns dCVA/dlambda. */
double oracle_cva(const double* ee, int n_dates, double dtau, double hazard, double recovery, double* dcva_dhazard)
{
    double cva = 0.0, d = 0.0;
    for (int j = 1; j < n_dates; ++j) {
        double t0 = (j - 1) * dtau, t1 = j * dtau;
        double e0 = exp(-hazard * t0), e1 = exp(-hazard * t1);
        cva += ee[j] * (e0 - e1);
        d += ee[j] * (-t0 * e0 + t1 * e1);
    }
    if (dcva_dhazard) *dcva_dhazard = (1.0 - recovery) * d;
    return (1.0 - recovery) * cva;
}

/* Per-path CVA contributions c_p = (1-R) sum_j w_j E_p(t_j); their mean is CVA. */
void oracle_cva_paths(const double* exposures, int n_paths, int n_tenor, int n_dates,
                      double dtau, double hazard, double recovery, double* out)
{
    for (int p = 0; p < n_paths; ++p) {
        double c = 0.0;
        for (int j = 1; j < n_dates; ++j) {
            double w = exp(-hazard * (j - 1) * dtau) - exp(-hazard * j * dtau);
            c += exposures[(size_t)p * n_tenor + j] * w;
        }
        out[p] = (1.0 - recovery) * c;
    }
}

/* Rank (1-based) of the q-quantile under the inverted-CDF definition. */
long oracle_quantile_rank(double q, long n)
{
    double x = q * (double)n - 1e-7;
    long k = (long)ceil(x);
    if (k < 1) k = 1;
    if (k > n) k = n;
    return k;
}

static int cmp_double(const void* a, const void* b)
{
    double x = *(const double*)a, y = *(const double*)b;
    return (x > y) - (x < y);
}

/* PFE_t = k-th smallest exposure across paths at tenor t, k = quantile rank. */
void oracle_pfe(const double* exposures, int n_paths, int n_tenor, int n_dates, double q, double* pfe)
{
    double* col = (double*)malloc(sizeof(double) * (size_t)n_paths);
    long k = oracle_quantile_rank(q, n_paths);
    for (int t = 0; t < n_dates; ++t) {
        for (int p = 0; p < n_paths; ++p) col[p] = exposures[(size_t)p * n_tenor + t];
        qsort(col, (size_t)n_paths, sizeof(double), cmp_double);
        pfe[t] = col[k - 1];
    }
    free(col);
}

/* ------------------------------------------------------------------------ */
/* Multi-threaded timing driver (CPU baseline): host Philox normals made     */
/* per path on the fly, the reference's per-path restatement, per-thread     */
/* partial EE sums combined in thread order.                                 */
/* ------------------------------------------------------------------------ */
typedef struct {
    const oracle_model* M;
    uint64_t seed, path0;
    long begin, end;
    double ee_sum[ORACLE_MAX_TENOR];
} mt_job;

static void* mt_worker(void* arg)
{
    mt_job* J = (mt_job*)arg;
    const oracle_model* M = J->M;
    double* nrm = (double*)malloc(sizeof(double) * (size_t)M->n_steps * 3);
    double e[ORACLE_MAX_TENOR], cf[ORACLE_MAX_TENOR];
    memset(J->ee_sum, 0, sizeof(J->ee_sum));
    for (long p = J->begin; p < J->end; ++p) {
        for (int n = 0; n < M->n_steps; ++n) normals3(J->seed, J->path0 + (uint64_t)p, (uint32_t)n, nrm + (size_t)n * 3);
        simulate_path(M, nrm, e, cf);
        for (int t = 0; t < M->nt; ++t) J->ee_sum[t] += e[t];
    }
    free(nrm);
    return NULL;
}

int oracle_run_mt(int n_tenor, double dtau, double dt, int n_steps,
                  const double* spot, const double* vol, const double* drift,
                  const double* accrual, double notional, double strike, double sign,
                  long n_paths, uint64_t seed, uint64_t path0, int n_threads, double* ee)
{
    oracle_model M;
    int rc = model_init(&M, n_tenor, dtau, dt, n_steps, spot, vol, drift, accrual, notional, strike, sign);
    if (rc) return rc;
    if (n_threads < 1) n_threads = 1;
    if (n_threads > 1024) n_threads = 1024;
    mt_job* jobs = (mt_job*)calloc((size_t)n_threads, sizeof(mt_job));
    pthread_t* th = (pthread_t*)calloc((size_t)n_threads, sizeof(pthread_t));
    for (int i = 0; i < n_threads; ++i) {
        jobs[i].M = &M; jobs[i].seed = seed; jobs[i].path0 = path0;
        jobs[i].begin = n_paths * i / n_threads;
        jobs[i].end = n_paths * (i + 1) / n_threads;
        pthread_create(&th[i], NULL, mt_worker, &jobs[i]);
    }
    for (int t = 0; t < n_tenor; ++t) ee[t] = 0.0;
    for (int i = 0; i < n_threads; ++i) {
        pthread_join(th[i], NULL);
        for (int t = 0; t < n_tenor; ++t) ee[t] += jobs[i].ee_sum[t];
    }
    for (int t = 0; t < n_tenor; ++t) ee[t] /= (double)n_paths;
    free(jobs);
    free(th);
    return 0;
}
