// hjm_eresp.h -- host interface of the FP64 Euler response form (hjm_eresp.cu).
#pragma once

#include "hjm_resp.cuh"

namespace hjm {

// Parameters of one launch: the path parameters (n_blocks = every date of the
// run), the block's moving-frame matrices, the basis centre, the window of
// dates this launch prices, and the table's slots per row (eresp_row).
// frame: the window's coefficient rows (launch_eresp_tables writes one set
// per window after the active prefixes, frame_index picks it).  renorm:
// renormalise the date slots' double-FP32 pairs every fourth step.
// Without it the low part of a pair gathers every rounding error of the high
// part, so that after n additions it is ~sqrt(n) ulps of the sum and rounds
// at ~n 2^-49 of the sum; that is negligible for the small remainder of a
// 20-date run, but not for the dates next to the last tenor (remainder and
// running sum a sizeable part of the curve over thousands of steps) nor for
// the residual terms, which the low parts accumulate (their running total
// sets the low parts' rounding unless it is moved into the high parts).
// Every fourth step keeps the low part within about two ulps of the sum.
// wnew_L: the predictor-corrector's source at the last tenor per unit of W
// after the step (gL = -c dtau^2; 0 for Euler).  Its term of a step enters
// the remainder after the step, so for the one date that samples the last
// tenor (tenor_L; with nt - 1 dates) the term of its own sampling step has
// lag -1, outside the table: the kernel adds it when it prices that date.
struct EulerRespParams {
    PathParams<double> P;
    BlockFrameN frame;
    double tau0;
    double wnew_L;
    int tenor_L;
    int win_lo, win_hi;
    int row;
    int renorm;
    int frame_index, n_frames;
};

// The parts' step of one window: NP parts, N's entries, B[c][k] = the
// loading of part c on factor k (sqrt(dt) times the coefficient of t^c of
// factor k, t = T - tau0), the basis centre tau0, and (NP = 4) sig0 =
// 3 (T_L - tau0), the cubic's share in the remainder's source: at the last
// tenor the polynomial is off by -c (P(T_L + dtau) - 2 P(T_L) + P(T_L - dtau))
// = kappa (x_2 + 3 (T_L - tau0) x_3), kappa = -2 c dtau^2.
struct EulerRespFrame {
    int np;
    PartsN n;
    double bm[4][kFactors];
    double tau0;
    double sig0;
};

// The frame of a window whose basis is centred at tau0: from svc [3][3], the
// quadratic loadings sqrt(dt) c_{k,d} of T^d, or, with cubic [3][4]
// (coefficients of (T - T_L)^d, unscaled) and their degrees, from the cubic;
// the polynomials re-expanded in powers of T - tau0 (a Taylor shift in FP64).
// degs: degs_pack of the factors' degrees.
// pc: the predictor-corrector's two-stage step on the parts (N's entry
// n02 = (c + c^2) dtau^2 instead of c dtau^2; svc then holds its N-projected
// loadings, quadratic only).
void eresp_make_frame(double dt, double dtau, int nt, const double (*svc)[3], const double* cubic,
                      const int* cubic_degs, double tau0, EulerRespFrame& fr, int& degs, bool pc = false);
// The basis centre of a window: the middle of its sampled tenors, where the
// polynomial's terms cancel least (at T_L the cubic's terms at the early
// tenors are ~30 times the net loading, and so are their rounding errors).
double eresp_window_centre(double dtau, int lo, int hi);
int eresp_row(int n_blocks);
// float4 entries of the table buffer: responses, active prefixes, then the
// frame coefficients of n_frames windows.  nres: factors with a residual (0;
// 2: factors 2 and 3; 3: all).
size_t eresp_table_elems(int stride, int n_blocks, int np, int nres, int n_frames);
// Build the table on the stream (clears the buffer first).  resid: the
// residual loadings sqrt(dt) (sigma_k - poly_k) [3][nt], or null; nres as
// above (with nres = 2 the first factor's residual is left out).
// pc: the predictor-corrector step's remainder responses (no residual).
cudaError_t launch_eresp_tables(int nt, double c, double dtau, int stride, int n_blocks, const EulerRespFrame* frames,
                                int n_frames, const double* resid, int nres, bool pc, float4* table, cudaStream_t s);
// The earliest date whose remainder terms the table's active prefixes can
// ever hold (n_blocks + 1 when none): the host's FP64 restatement of
// eresp_active_kernel's test at half its thresholds, so that it never
// misses a date the device counts.  With a residual (nres > 0), 2: the
// residual loadings reach every tenor.
// pc: the predictor-corrector step's table (eresp_table_pc_kernel).
int eresp_first_active_date(int nt, double c, int stride, int n_blocks, int nres, bool pc = false);
// The predictor-corrector's remainder source per unit W and step (the scale
// of its table's entries, as kappa = -2 c dtau^2 is the Euler step's).
double eresp_kappa_pc(double c, double dtau);
// The residual factors a table needs: 0 without a residual, 2 when the first
// factor's residual is at most 2^-44 of its scale (an exact constant, as the
// reference table's first factor), else 3.
int eresp_residual_factors(const double* resid, const double* vol, int nt);
// The windows of a run of n_blocks dates, latest first (lo, hi, ns may be
// null): their number.  A window needs a register slot only for its dates
// that can be active, from first_active (eresp_first_active_date; 2 for
// every date) on; earlier dates, never reached by the remainder, are priced
// with no slot.  From the latest date down, a window takes every remaining
// date when those that can be active number at most kRespSlots, else the
// kRespSlots latest (a window reaching date 2 takes date 1 too).  ns: the
// slots the window's kernel holds, 12, 16, 20 or 24, at least its active ones.
// max_slots: the dates a window holds (eresp_window_dates; the
// volatility-table response form takes 16).
int eresp_windows(int n_blocks, int first_active, int* lo, int* hi, int* ns, int max_slots = kRespSlots);
// The dates a window of the response form holds: kRespSlots, or 16 with a
// residual table (every date still to be sampled is active; 16 register slots
// fit 128 registers without spills, 8 CTAs per SM).
inline int eresp_window_dates(int nres) { return nres > 0 ? 16 : kRespSlots; }
// One launch per window, latest first, window w with frame w (its centre in
// frames[w].tau0).  degs: the factors' degrees
// (degs_pack); nres: the table's residual factors; first_active: as
// eresp_windows (the frames' windows); carry [2][n_paths] doubles when the
// run has more than one window.  *launches: kernels enqueued.
cudaError_t launch_path_fp64_eresp(const EulerRespParams& base, const EulerRespFrame* frames, int degs, int nres,
                                   const float4* table, int first_active,
                                   const double* ext, double* partials, double* estore, double* carry,
                                   cudaStream_t s, int* launches);
// The largest dynamic shared memory of the run's launches.
size_t eresp_max_smem(int n_blocks, int np, int stride, int first_active, int nres);

}  // namespace hjm
