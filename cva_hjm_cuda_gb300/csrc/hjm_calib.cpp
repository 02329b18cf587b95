// hjm_calib.cpp -- the market-input step before the path: volatility factors
// of the HJM model from historical forward curves.
//
// The reference hard-codes the output of this step (the 3 x 51 volatility
// table of simulation_gpu_testing.cpp:47-63, and the drift table it implies)
// and lists the calibration as a to-do (doc/TODO:13).  The published HJM
// recipe it stands for: principal components of the covariance of the daily
// changes of the forward curve, annualised; factor k's volatility is
// sqrt(lambda_k) times its eigenvector; each factor is then smoothed by a
// low-degree polynomial in the tenor (the reference's factors are degree 0, 1
// and 2).  The whole step is O(n_obs n_tenor^2 + n_tenor^3) floating-point
// work (about 10^7 operations for ten years of daily curves): host C++ in
// FP64, no GPU involved.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "../../include/hjm_cva.h"

namespace hjm {
void set_thread_error(const char* msg);  // hjm_capi.cu
}

namespace {

hjm_status calib_fail(hjm_status st, const char* msg)
{
    hjm::set_thread_error(msg);
    return st;
}

// Cyclic Jacobi eigen-decomposition of the symmetric n x n matrix a (row
// major, destroyed): eigenvalues to w, eigenvectors to the columns of v.
// Rotations zero one off-diagonal element at a time (Golub & Van Loan,
// "Matrix Computations", sec. 8.5); sweeps until the off-diagonal mass is
// below 1e-30 of the diagonal's, at most 100 sweeps.
bool jacobi_eigen(int n, std::vector<double>& a, std::vector<double>& w, std::vector<double>& v)
{
    v.assign((size_t)n * n, 0.0);
    for (int i = 0; i < n; ++i) v[(size_t)i * n + i] = 1.0;
    auto A = [&](int i, int j) -> double& { return a[(size_t)i * n + j]; };
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, diag = 0.0;
        for (int i = 0; i < n; ++i) {
            diag += A(i, i) * A(i, i);
            for (int j = i + 1; j < n; ++j) off += A(i, j) * A(i, j);
        }
        if (off <= 1e-30 * diag || off == 0.0) {
            w.resize(n);
            for (int i = 0; i < n; ++i) w[i] = A(i, i);
            return true;
        }
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A(p, q);
                if (apq == 0.0) continue;
                const double theta = (A(q, q) - A(p, p)) / (2.0 * apq);
                const double t = (theta >= 0.0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {  // columns p, q
                    const double akp = A(k, p), akq = A(k, q);
                    A(k, p) = c * akp - s * akq;
                    A(k, q) = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {  // rows p, q
                    const double apk = A(p, k), aqk = A(q, k);
                    A(p, k) = c * apk - s * aqk;
                    A(q, k) = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = v[(size_t)k * n + p], vkq = v[(size_t)k * n + q];
                    v[(size_t)k * n + p] = c * vkp - s * vkq;
                    v[(size_t)k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    return false;
}

// Least-squares coefficients of y on 1, T, ..., T^deg (deg <= 2) by modified
// Gram-Schmidt on the columns (well conditioned for T up to 31.5).
void poly_fit(const double* y, const double* T, int n, int deg, double* coef)
{
    const int m = deg + 1;
    std::vector<double> q((size_t)m * n), r((size_t)m * m, 0.0);
    for (int d = 0; d < m; ++d)
        for (int i = 0; i < n; ++i) q[(size_t)d * n + i] = std::pow(T[i], d);
    for (int d = 0; d < m; ++d) {
        double* qd = &q[(size_t)d * n];
        for (int e = 0; e < d; ++e) {
            const double* qe = &q[(size_t)e * n];
            double dot = 0.0;
            for (int i = 0; i < n; ++i) dot += qe[i] * qd[i];
            r[(size_t)e * m + d] = dot;
            for (int i = 0; i < n; ++i) qd[i] -= dot * qe[i];
        }
        double nrm = 0.0;
        for (int i = 0; i < n; ++i) nrm += qd[i] * qd[i];
        nrm = std::sqrt(nrm);
        r[(size_t)d * m + d] = nrm;
        for (int i = 0; i < n; ++i) qd[i] /= nrm;
    }
    double z[3] = {0.0, 0.0, 0.0};
    for (int d = 0; d < m; ++d) {
        double dot = 0.0;
        for (int i = 0; i < n; ++i) dot += q[(size_t)d * n + i] * y[i];
        z[d] = dot;
    }
    for (int d = m - 1; d >= 0; --d) {  // back substitution R c = z
        double s = z[d];
        for (int e = d + 1; e < m; ++e) s -= r[(size_t)d * m + e] * coef[e];
        coef[d] = s / r[(size_t)d * m + d];
    }
    for (int d = m; d < 3; ++d) coef[d] = 0.0;
}

}  // namespace

extern "C" hjm_status hjm_calibrate_pca(const double* curves, int32_t n_obs, int32_t n_tenor, double dtau,
                                        double obs_per_year, int32_t n_factor, double* vol_out,
                                        double* eigval_out, double* coef_out, double* explained_out)
{
    if (!curves || !vol_out) return calib_fail(HJM_ERR_INVALID_ARGUMENT, "curves and vol_out must not be null");
    if (n_factor != HJM_N_FACTOR) return calib_fail(HJM_ERR_UNSUPPORTED, "the model has 3 factors");
    if (n_tenor < n_factor || n_tenor > HJM_MAX_TENOR)
        return calib_fail(HJM_ERR_INVALID_ARGUMENT, "n_tenor outside [3, HJM_MAX_TENOR]");
    if (n_obs < 3) return calib_fail(HJM_ERR_INVALID_ARGUMENT, "need at least 3 curves (2 changes)");
    if (!(dtau > 0.0) || !(obs_per_year > 0.0) || !std::isfinite(dtau) || !std::isfinite(obs_per_year))
        return calib_fail(HJM_ERR_INVALID_ARGUMENT, "dtau and obs_per_year must be finite and > 0");
    const int n = n_tenor, m = n_obs - 1;
    for (size_t i = 0; i < (size_t)n_obs * n; ++i)
        if (!std::isfinite(curves[i])) return calib_fail(HJM_ERR_INVALID_ARGUMENT, "curves must be finite");

    // changes, their means, and the annualised sample covariance
    std::vector<double> dx((size_t)m * n), mean(n, 0.0);
    for (int j = 0; j < m; ++j)
        for (int t = 0; t < n; ++t) {
            const double d = curves[(size_t)(j + 1) * n + t] - curves[(size_t)j * n + t];
            dx[(size_t)j * n + t] = d;
            mean[t] += d;
        }
    for (int t = 0; t < n; ++t) mean[t] /= m;
    std::vector<double> cov((size_t)n * n, 0.0);
    for (int j = 0; j < m; ++j) {
        const double* r = &dx[(size_t)j * n];
        for (int a = 0; a < n; ++a) {
            const double ra = r[a] - mean[a];
            for (int b = a; b < n; ++b) cov[(size_t)a * n + b] += ra * (r[b] - mean[b]);
        }
    }
    const double scale = obs_per_year / (double)(m - 1);
    double trace = 0.0;
    for (int a = 0; a < n; ++a)
        for (int b = a; b < n; ++b) {
            const double c = cov[(size_t)a * n + b] * scale;
            cov[(size_t)a * n + b] = c;
            cov[(size_t)b * n + a] = c;
            if (a == b) trace += c;
        }
    if (!(trace > 0.0)) return calib_fail(HJM_ERR_INVALID_ARGUMENT, "the curves do not change");

    std::vector<double> w, v;
    if (!jacobi_eigen(n, cov, w, v)) return calib_fail(HJM_ERR_UNSUPPORTED, "eigen-decomposition did not converge");
    std::vector<int> order(n);
    for (int i = 0; i < n; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) { return w[x] > w[y]; });

    std::vector<double> T(n);
    for (int t = 0; t < n; ++t) T[t] = dtau * t;
    double expl = 0.0;
    for (int k = 0; k < n_factor; ++k) {
        const int col = order[k];
        const double lam = std::max(w[col], 0.0);
        expl += lam;
        // sign: the component of largest magnitude is positive
        int imax = 0;
        for (int t = 1; t < n; ++t)
            if (std::fabs(v[(size_t)t * n + col]) > std::fabs(v[(size_t)imax * n + col])) imax = t;
        const double sgn = v[(size_t)imax * n + col] < 0.0 ? -1.0 : 1.0;
        const double sl = std::sqrt(lam) * sgn;
        for (int t = 0; t < n; ++t) vol_out[(size_t)k * n + t] = sl * v[(size_t)t * n + col];
        if (eigval_out) eigval_out[k] = lam;
        if (coef_out) poly_fit(vol_out + (size_t)k * n, T.data(), n, std::min(k, 2), coef_out + 3 * k);
    }
    if (explained_out) *explained_out = expl / trace;
    return HJM_OK;
}
