"""CPU checks of the FP64 response form's algorithm (no GPU).

The response form carries the remainder hc of the polynomial decomposition,
driven by kappa W at the last tenor and convected upwind, as impulse-response
sums at the sampled tenors: for date j, hc at its sampling step and the
running sum of hc, both sum_n coef(lag) W_{n-1}.  Restated here in numpy, as
eresp_table_kernel (eresp_table_pc_kernel for the predictor-corrector) and
path_kernel_fp64_eresp compute them (the Euler prefix rule of
eresp_active_kernel is in test_cubic_windows.py):

* the table: entry (row b*stride + s, slot B - j) holds kappa G_j(lag) and
  kappa CG_j(lag), lag = (j - b) stride - 1 - s, every lag of every date in
  exactly one entry;
* the active prefix: at step s of block b the slots 0 .. n_act - 1 with
  q_min = ceil((s + 1 + L - b) / (stride + 1)) cover every nonzero entry;
* the sums equal the direct recursion hc <- A hc + kappa W e_L to rounding;
* the double-FP32 arithmetic (truncation split of W, exact leading product,
  two-sum) stays within ~1e-12 of the FP64 sums, and the split within 2^-47.
"""
from __future__ import annotations

import struct

import numpy as np
import pytest

ROW = 24  # table row width (slots)


def response_table(nt, stride, B, c, dtau):
    L = nt - 1
    kappa = -2.0 * c * dtau * dtau
    tab = np.zeros((B * stride * ROW, 2))
    written = np.zeros(B * stride * ROW, dtype=int)
    v = np.zeros(nt)
    v[L] = 1.0
    cum = np.zeros(nt)
    for m in range((B - 1) * stride):
        cum = cum + v
        for t in range(2, B + 1):
            q = m // stride + 1
            b = t - q
            if b >= 1:
                idx = (b * stride + (q * stride - 1 - m)) * ROW + (B - t)
                tab[idx] = (kappa * v[t], kappa * cum[t])
                written[idx] += 1
        vn = v.copy()
        vn[:L] = v[:L] + c * (v[1:] - v[:L])
        vn[L] = v[L] + c * (v[L] - v[L - 1])
        v = vn
    return tab, written, kappa


def n_active(s, b, B, L, stride):
    q_min = (s + 1 + L - b + stride) // (stride + 1)
    return B - b - q_min + 1


SHAPES = [(51, 50, 20, 0.02), (61, 50, 20, 0.02), (51, 25, 24, 0.04), (51, 100, 10, 0.01), (51, 10, 5, 0.1)]


@pytest.mark.parametrize("nt,stride,B,c", SHAPES)
def test_table_covers_every_lag_once_and_prefix_holds_the_nonzeros(nt, stride, B, c):
    tab, written, _ = response_table(nt, stride, B, c, 0.5)
    L = nt - 1
    assert written.max() <= 1
    for b in range(1, B):
        for s in range(stride):
            n_act = n_active(s, b, B, L, stride)
            assert n_act <= 23
            for r in range(ROW):
                idx = (b * stride + s) * ROW + r
                live = r < B - b  # date j = B - r > b
                assert written[idx] == (1 if live and B - r >= 2 else 0)
                if r >= max(n_act, 0):
                    assert tab[idx, 0] == 0.0 and tab[idx, 1] == 0.0, (b, s, r)


@pytest.mark.parametrize("nt,stride,B,c", SHAPES)
def test_value_prefix_drops_only_vanishing_terms(nt, stride, B, c):
    """The kernels' prefix from the table's values never exceeds the
    closed-form one, and the terms it drops (near the transport front) add up,
    over all its rows (at most 2,400 here), to less than rows x 2^-70 of the
    date's largest coefficient per unit |W|: below 2^-58, far under the
    double-FP32 sums' own 2^-48 rounding."""
    tab, _, _ = response_table(nt, stride, B, c, 0.5)
    L = nt - 1
    pre = active_prefix(tab, B, stride)
    T = tab.reshape(B * stride, ROW, 2)
    dropped = np.zeros((ROW, 2))
    for b in range(1, B):
        for s in range(stride):
            n = b * stride + s
            assert pre[n] <= max(n_active(s, b, B, L, stride), 0)
            # (entries that are zero in FP32 are zeros of the kernels' table anyway)
            tail = T[n, pre[n]:]
            dropped[pre[n]:] += np.where(tail.astype(np.float32) != 0, np.abs(tail), 0.0)
    big = np.abs(T).max(axis=0)
    assert np.all(dropped <= B * stride * 2.0 ** -70 * big + 1e-300)
    if (nt, stride, B) == (51, 50, 20):
        assert pre[stride:].mean() < 0.9 * np.mean([max(n_active(s, b, B, L, stride), 0)
                                                    for b in range(1, B) for s in range(stride)])


def active_prefix(tab, B, stride):
    """An earlier, stricter prefix rule: per row, the slots up to the last
    whose coefficient or running-sum coefficient (FP32 hi part) is nonzero
    and at least 2^-70 of its slot's largest over all rows (the kernels now
    cut at FP64's unit roundoff of the unit response, eresp_active_kernel)."""
    T = tab.reshape(B * stride, ROW, 2).astype(np.float32)
    a = np.abs(T)
    thr = (a.max(axis=0) * np.float32(2.0 ** -70)).astype(np.float32)
    sig = ((T != 0) & (a >= thr)).any(axis=2)
    return np.where(sig.any(axis=1), ROW - np.argmax(sig[:, ::-1], axis=1), 0)


def _direct_and_response(nt, stride, B, c, dtau, W, df=False, cutoff=False):
    tab, _, kappa = response_table(nt, stride, B, c, dtau)
    prefix = active_prefix(tab, B, stride) if cutoff else None
    L = nt - 1
    acc = np.zeros((ROW, 2))
    dfa = [[DF(), DF()] for _ in range(ROW)]
    hc = np.zeros(nt)
    hsum = np.zeros(nt)
    got, want = {}, {}
    w = 0.0
    for b in range(1, B):
        for s in range(stride):
            n = b * stride + s
            n_act = prefix[n] if cutoff else n_active(s, b, B, L, stride)
            wh, wl = split_f64(w)
            for r in range(max(n_act, 0)):
                k = tab[(b * stride + s) * ROW + r]
                acc[r] += k * w
                if df:
                    for q in range(2):
                        dfa[r][q].add(k[q], wh, wl)
            hn = hc.copy()
            hn[:L] = hc[:L] + c * (hc[1:] - hc[:L])
            hn[L] = hc[L] + c * (hc[L] - hc[L - 1]) + kappa * w
            hc = hn
            hsum += hc
            w = W[n]
        j = b + 1
        r = B - j
        want[j] = (hc[j], hsum[j])
        got[j] = tuple(dfa[r][q].value() for q in range(2)) if df else (acc[r, 0], acc[r, 1])
    return got, want


def _rel(a, b):
    return abs(a - b) / abs(b) if b != 0.0 else abs(a)


@pytest.mark.parametrize("cutoff", [False, True], ids=["closed-form-prefix", "value-prefix"])
@pytest.mark.parametrize("nt,stride,B,c", SHAPES[:4])
def test_response_sums_equal_the_convected_remainder(nt, stride, B, c, cutoff):
    rng = np.random.default_rng(7)
    W = np.cumsum(rng.normal(size=B * stride)) * 1e-5
    got, want = _direct_and_response(nt, stride, B, c, 0.5, W, cutoff=cutoff)
    big = np.abs(response_table(nt, stride, B, c, 0.5)[0].reshape(B * stride, ROW, 2)).max(axis=0)
    for j in got:
        for q in range(2):
            # the value prefix drops terms below rows x 2^-70 of the date's largest
            # per unit |W|, and coefficients below FP32's range (the table's
            # FP32 pairs hold them as zeros; 1e-30 is far below the curve's ulp)
            floor = B * stride * 2.0 ** -70 * big[B - j, q] * np.max(np.abs(W)) + 1e-30 if cutoff else 0.0
            assert abs(got[j][q] - want[j][q]) <= 1e-12 * abs(want[j][q]) + floor, (j, q, got[j][q], want[j][q])


# --- double-FP32 arithmetic, as the kernel's split_f64 / df_acc -------------
_f32 = np.float32


def _bits_f32(u):
    return struct.unpack("<f", struct.pack("<I", u))[0]


def split_f64(d):
    u = struct.unpack("<Q", struct.pack("<d", float(d)))[0]
    top = u >> 32
    sign = top & 0x80000000
    eh = ((top >> 20) & 0x7FF) - 1023 + 127
    if eh <= 0:
        return _f32(_bits_f32(sign)), _f32(_bits_f32(sign))
    if eh > 254:
        return _f32(_bits_f32(sign | 0x7F7FFFFF)), _f32(_bits_f32(sign))
    hi = _f32(_bits_f32(sign | (eh << 23) | ((u >> 29) & 0x7FFFFF)))
    r = u & 0x1FFFFFFF
    scale = _f32(_bits_f32((eh - 52) << 23)) if eh > 52 else _f32(0.0)
    lo_abs = _f32(_f32(r) * scale)
    lo = _f32(_bits_f32(sign | struct.unpack("<I", struct.pack("<f", lo_abs))[0]))
    return hi, lo


def _fma32(a, b, c):
    # float32 a*b is exact in float64; one float64 rounding before the float32 one
    return _f32(np.float64(a) * np.float64(b) + np.float64(c))


class DF:
    """One lane of the kernel's (A, Al) accumulator."""

    def __init__(self):
        self.A = _f32(0.0)
        self.Al = _f32(0.0)

    def add(self, k, wh, wl):
        kh = _f32(k)
        kl = _f32(k - np.float64(kh))
        p = _f32(kh * wh)
        e = _fma32(kh, wh, -p)
        e = _fma32(kh, wl, e)
        e = _fma32(kl, wh, e)
        s = _f32(self.A + p)
        bp = _f32(s - self.A)
        ap = _f32(s - bp)
        err = _f32(_f32(self.A - ap) + _f32(p - bp))
        self.Al = _f32(self.Al + _f32(err + e))
        self.A = s

    def value(self):
        return np.float64(self.A) + np.float64(self.Al)


def test_split_is_within_2_pow_47():
    rng = np.random.default_rng(0)
    d = rng.normal(size=4000) * 10.0 ** rng.uniform(-20, 3, size=4000)
    for x in d:
        hi, lo = split_f64(x)
        assert abs(np.float64(hi) + np.float64(lo) - x) <= 2.0**-47 * abs(x)
        assert abs(np.float64(hi)) <= abs(x)
    assert split_f64(0.0) == (0.0, 0.0)
    hi, lo = split_f64(1e-30)  # below 2^-74: the low part is dropped, hi truncated
    assert lo == 0.0 and abs(np.float64(hi) - 1e-30) <= 2.0**-23 * 1e-30


@pytest.mark.parametrize("nt,stride,B,c", [(51, 50, 24, 0.02), (51, 25, 24, 0.04), (51, 50, 20, 0.02)])
def test_double_fp32_sums_track_fp64_sums(nt, stride, B, c):
    """The most dates the form takes (24, the remainder nearest the transport
    front), with a curvature random walk five times the reference market's.
    Terms whose coefficient lies below FP32's range (under ~1e-38: the far
    tail of the transport at early dates) come out as zero; the absolute
    floor 1e-30 is far below the curve's FP64 ulp (~3e-18)."""
    rng = np.random.default_rng(1)
    W = np.cumsum(rng.normal(size=B * stride)) * np.sqrt(c * 0.5) * 2e-5 * 5
    got, want = _direct_and_response(nt, stride, B, c, 0.5, W, df=True)
    for j in got:
        for q in range(2):
            assert abs(got[j][q] - want[j][q]) <= 2e-12 * abs(want[j][q]) + 1e-30, (j, q, got[j][q], want[j][q])
    assert abs(want[B][0]) > 1e-7  # the last date's remainder is well inside FP32's range


# --- predictor-corrector -----------------------------------------------------
def pc_step(v, c):
    """A2: three-point stencil a0, a1, a2 below L-1; Euler rows at L-1, L."""
    L = v.size - 1
    a0, a1, a2 = 1 - c + c * c / 2, c - c * c, c * c / 2
    vn = v.copy()
    vn[:L - 1] = a0 * v[:L - 1] + a1 * v[1:L] + a2 * v[2:L + 1]
    vn[L - 1] = v[L - 1] + c * (v[L] - v[L - 1])
    vn[L] = v[L] + c * (v[L] - v[L - 1])
    return vn


def pc_sources(c, dtau):
    return -c * c * dtau * dtau, -(2 * c + c * c) * dtau * dtau, -c * dtau * dtau  # wL1, wL, gL


def response_table_pc(nt, stride, B, c, dtau):
    """As eresp_table_pc_kernel: the coefficient of the old W at lag l is
    H1(l) + H2(l+1), H1 = wL1 G1 + (wL - gL) G2, H2 = gL G2."""
    L = nt - 1
    wL1, wL, gL = pc_sources(c, dtau)
    w0, w1, w2 = wL1, wL - gL, gL
    tab = np.zeros((B * stride * ROW, 2))
    written = np.zeros(B * stride * ROW, dtype=int)
    g1 = np.zeros(nt)
    g1[L - 1] = 1.0
    g2 = np.zeros(nt)
    g2[L] = 1.0
    cg1, cg2 = np.zeros(nt), np.zeros(nt)
    h1p, ch1p = np.zeros(nt), np.zeros(nt)
    for m in range((B - 1) * stride + 1):
        cg1, cg2 = cg1 + g1, cg2 + g2
        if m >= 1:
            l = m - 1
            for t in range(2, B + 1):
                q = l // stride + 1
                b = t - q
                if b >= 1:
                    idx = (b * stride + (q * stride - 1 - l)) * ROW + (B - t)
                    tab[idx] = (h1p[t] + w2 * g2[t], ch1p[t] + w2 * cg2[t])
                    written[idx] += 1
        h1p, ch1p = w0 * g1 + w1 * g2, w0 * cg1 + w1 * cg2
        g1, g2 = pc_step(g1, c), pc_step(g2, c)
    return tab, written


def n_active_pc(s, b, B, L, stride):
    q_min = max(1, -(-(L - b + 2 * s) // (2 * stride + 1)))
    return B - b - q_min + 1


@pytest.mark.parametrize("nt,stride,B,c", SHAPES)
def test_pc_table_covers_every_lag_once_and_prefix_holds_the_nonzeros(nt, stride, B, c):
    tab, written = response_table_pc(nt, stride, B, c, 0.5)
    L = nt - 1
    assert written.max() <= 1
    for b in range(1, B):
        for s in range(stride):
            n_act = n_active_pc(s, b, B, L, stride)
            for r in range(ROW):
                idx = (b * stride + s) * ROW + r
                live = r < B - b
                assert written[idx] == (1 if live and B - r >= 2 else 0)
                if r >= max(n_act, 0):
                    assert tab[idx, 0] == 0.0 and tab[idx, 1] == 0.0, (b, s, r)


@pytest.mark.parametrize("nt,stride,B,c", SHAPES[:4])
def test_pc_response_sums_equal_the_convected_remainder(nt, stride, B, c):
    """The remainder of the predictor-corrector's polynomial form, driven at
    L-1 by wL1 W and at L by wL W + gL gamma (gamma the step's curvature noise,
    W the curvature before the step), against the response sums of the old W."""
    dtau = 0.5
    tab, _ = response_table_pc(nt, stride, B, c, dtau)
    wL1, wL, gL = pc_sources(c, dtau)
    L = nt - 1
    rng = np.random.default_rng(3)
    acc = np.zeros((ROW, 2))
    hc, hsum = np.zeros(nt), np.zeros(nt)
    W = 0.0
    for b in range(1, B):
        for s in range(stride):
            n_act = n_active_pc(s, b, B, L, stride)
            for r in range(max(n_act, 0)):
                acc[r] += tab[(b * stride + s) * ROW + r] * W
            gam = rng.normal() * 1e-5
            hn = pc_step(hc, c)
            hn[L - 1] += wL1 * W
            hn[L] += wL * W + gL * gam
            hc = hn
            hsum += hc
            W += gam
        j = b + 1
        for got, want in ((acc[B - j, 0], hc[j]), (acc[B - j, 1], hsum[j])):
            assert abs(got - want) <= 1e-12 * abs(want) + 1e-300, (j, got, want)


def test_pc_date_at_the_last_tenor_takes_the_lag_minus_one_term():
    """With as many dates as tenors after the first (B = L), the date that
    samples the last tenor also takes gL times W after its own sampling step
    (the step's curvature noise enters at L after the step, a lag -1 term the
    table cannot hold); path_kernel_fp64_eresp adds it when it prices that
    date.  Value and running sum against the direct recursion."""
    nt, stride, c, dtau = 11, 10, 0.1, 0.5
    L = B = nt - 1
    tab, _ = response_table_pc(nt, stride, B, c, dtau)
    wL1, wL, gL = pc_sources(c, dtau)
    rng = np.random.default_rng(11)
    acc = np.zeros((ROW, 2))
    hc, hsum = np.zeros(nt), np.zeros(nt)
    W = 0.0
    for b in range(1, B):
        for s in range(stride):
            for r in range(B - b):
                acc[r] += tab[(b * stride + s) * ROW + r] * W
            gam = rng.normal() * 1e-5
            hn = pc_step(hc, c)
            hn[L - 1] += wL1 * W
            hn[L] += wL * W + gL * gam
            hc = hn
            hsum += hc
            W += gam
        j = b + 1
        got_v, got_s = acc[B - j, 0], acc[B - j, 1]
        if j == L:
            got_v, got_s = got_v + gL * W, got_s + gL * W
        for got, want in ((got_v, hc[j]), (got_s, hsum[j])):
            assert abs(got - want) <= 1e-12 * abs(want) + 1e-300, (j, got, want)


def eresp_prefix_pc(tab, B, stride, c, dtau):
    """As eresp_active_kernel on the predictor-corrector's table: the slots up
    to the last whose FP32 coefficient reaches 2^-53 |kappa_pc| or running-sum
    coefficient 2^-53 |kappa_pc| times the date's sampling step, kappa_pc =
    -(2c + 2c^2) dtau^2 (the step's source per unit W)."""
    kappa = -(2 * c + 2 * c * c) * dtau * dtau
    T = tab.reshape(B * stride, ROW, 2)
    a = np.abs(T.astype(np.float32))
    tg = np.float32(abs(kappa)) * np.float32(2.0 ** -53)
    dates = np.maximum(B - np.arange(ROW), 1)
    tcg = (tg * (dates * stride).astype(np.float32)).astype(np.float32)
    sig = ((a[:, :, 0] != 0) & (a[:, :, 0] >= tg)) | ((a[:, :, 1] != 0) & (a[:, :, 1] >= tcg[None, :]))
    return np.where(sig.any(axis=1), ROW - np.argmax(sig[:, ::-1], axis=1), 0), kappa


@pytest.mark.parametrize("nt,stride,B,c", SHAPES)
def test_pc_eresp_prefix_drops_only_terms_below_the_unit_roundoff(nt, stride, B, c):
    """The response kernel's prefix on the predictor-corrector's table skips,
    per date, terms that sum to less than 32 x 2^-53 |kappa_pc| per unit |W|
    (per sampling step for the running sum), as on the Euler step's."""
    tab, _ = response_table_pc(nt, stride, B, c, 0.5)
    pre, kappa = eresp_prefix_pc(tab, B, stride, c, 0.5)
    T = tab.reshape(B * stride, ROW, 2)
    for t in range(2, B + 1):
        r = B - t
        rows = np.arange(stride, t * stride)
        dropped = rows[pre[rows] <= r]
        assert np.abs(T[dropped, r, 0]).sum() <= 32 * 2.0 ** -53 * abs(kappa), t
        assert np.abs(T[dropped, r, 1]).sum() <= 32 * 2.0 ** -53 * abs(kappa) * t * stride, t


# --- volatility-table step: the whole stochastic curve in factor responses ---
def euler_step(v, c):
    L = v.size - 1
    vn = v.copy()
    vn[:L] = v[:L] + c * (v[1:] - v[:L])
    vn[L] = v[L] + c * (v[L] - v[L - 1])
    return vn


@pytest.mark.parametrize("scheme", ["euler", "pc"])
@pytest.mark.parametrize("nt,stride,B,c", SHAPES[:4])
def test_vol_table_response_sums_equal_the_direct_recursion(scheme, nt, stride, B, c):
    """As response_table_vol_kernel and path_kernel_fp64_vresp: entry (step,
    slot B - j, factor k) = (R_jk, CR_jk) at lag l, R_jk(l) = (A^l S_k)[j]; the
    sums over steps of R phi equal h <- A h + S phi at the dates."""
    step = pc_step if scheme == "pc" else euler_step
    L = nt - 1
    rng = np.random.default_rng(11)
    S = rng.uniform(0.001, 0.01, size=(3, nt)) * np.sqrt(c * 0.5)
    tab = np.zeros((B * stride * ROW, 3, 2))
    v = S.copy()
    cum = np.zeros_like(S)
    for m in range((B - 1) * stride):
        cum = cum + v
        for t in range(2, B + 1):
            q = m // stride + 1
            b = t - q
            if b >= 1:
                tab[(b * stride + (q * stride - 1 - m)) * ROW + (B - t)] = np.stack([v[:, t], cum[:, t]], axis=1)
        v = np.stack([step(v[k], c) for k in range(3)])
    acc = np.zeros((ROW, 2))
    h, hsum = np.zeros(nt), np.zeros(nt)
    for b in range(1, B):
        for s in range(stride):
            phi = rng.normal(size=3)
            for r in range(B - b):
                e = tab[(b * stride + s) * ROW + r]
                acc[r] += e.T @ phi
            h = step(h, c) + S.T @ phi
            hsum += h
        j = b + 1
        for got, want in ((acc[B - j, 0], h[j]), (acc[B - j, 1], hsum[j])):
            assert abs(got - want) <= 1e-12 * abs(want) + 1e-300, (j, got, want)


# --- the parts S, U, W in the moving frame (path_kernel_fp64_eresp) ---
SVC_TRI = np.sqrt(0.01) * np.array([[0.0064, 0.0, 0.0], [-0.0036, 0.0004, 0.0], [0.0020, -0.0006, 0.00002]])
SVC_GEN = SVC_TRI + np.sqrt(0.01) * np.array([[0.0, 1e-4, 2e-6], [0.0, 0.0, -3e-6], [0.0, 0.0, 0.0]])


def state_coefs(stride, n01, n02, n12, svc):
    """As eresp_coef_kernel: row s < stride (the step within a block) holds
    C(s) = M^-(s+1) B and G(s) = Q(s) C(s), B[c][k] = svc[k][c], M = I + N,
    N = [[0, n01, n02], [0, 0, n12], [0, 0, 0]]."""
    Bm = np.asarray(svc, dtype=np.float64).T
    nn = n01 * n12
    rows = {}
    for m in range(stride):
        kk, q = m + 1.0, float(m)
        minv = np.array([[1.0, -kk * n01, -kk * n02 + 0.5 * kk * (kk + 1.0) * nn], [0.0, 1.0, -kk * n12],
                         [0.0, 0.0, 1.0]])
        h = 0.5 * q * (q + 1.0)
        Q = np.array([[q, h * n01, h * n02 + (q + 1.0) * q * (q - 1.0) / 6.0 * nn], [0.0, q, h * n12],
                      [0.0, 0.0, q]])
        C = minv @ Bm
        rows[m] = (C, Q @ C)
    return rows


def block_end(y, v, z, a, n01, n02, n12):
    """As frame_block_end after a block of a steps: x = M^a y and
    Z + Q(a) y - v."""
    ha, nn = 0.5 * a * (a + 1.0), n01 * n12
    m02 = 0.5 * a * (a - 1.0) * nn + a * n02
    q02 = (a + 1.0) * a * (a - 1.0) / 6.0 * nn + ha * n02
    x = (y[0] + a * n01 * y[1] + m02 * y[2], y[1] + a * n12 * y[2], y[2])
    zn = (z[0] + (a * y[0] + ha * n01 * y[1] + q02 * y[2] - v[0]),
          z[1] + (a * y[1] + ha * n12 * y[2] - v[1]), z[2] + (a * y[2] - v[2]))
    return np.array(x), np.array(zn)


class DFW(DF):
    def add_exact(self, k, w):
        """As df_acc_w: w exact in FP32."""
        kh = _f32(k)
        kl = _f32(k - np.float64(kh))
        p = _f32(kh * w)
        e = _fma32(kh, w, -p)
        e = _fma32(kl, w, e)
        s = _f32(self.A + p)
        bp = _f32(s - self.A)
        ap = _f32(s - bp)
        err = _f32(_f32(self.A - ap) + _f32(p - bp))
        self.Al = _f32(self.Al + _f32(err + e))
        self.A = s

    def renorm(self):
        """As df_renorm (fast two-sum)."""
        s = _f32(self.A + self.Al)
        self.Al = _f32(self.Al - _f32(s - self.A))
        self.A = s


def _moving_frame_errors(svc, stride, B, dt, dtau, seed, df, scheme="euler"):
    """The parts and their running sums at the dates from the block-anchored
    moving frame (FP64 or the kernel's double-FP32) against the FP64
    recursion x <- M x + B phi of the scheme's step on a quadratic (Euler, or
    the predictor-corrector's (c + c^2) dtau^2 coupling of S to W); errors
    relative to the sum of the magnitudes of the terms of S + U tau + W tau^2
    at the date's tenor."""
    c = dt / dtau
    n01, n12 = c * dtau, 2.0 * c * dtau
    n02 = (c + c * c) * dtau * dtau if scheme == "pc" else c * dtau * dtau
    rows = state_coefs(stride, n01, n02, n12, svc)
    rng = np.random.default_rng(seed)
    phi = rng.normal(size=(B * stride, 3)).astype(np.float32)
    x = np.zeros(3)
    zsum = np.zeros(3)  # sum of the evolved parts
    xm, zm = np.zeros(3), np.zeros(3)  # the kernel's FP64 values between blocks
    errs = []
    for b in range(1, B):
        y, v = xm.copy(), np.zeros(3)
        acc = [[DFW(), DFW()] for _ in range(3)]
        for cc in range(3):  # the re-anchored accumulators: x rounded to an FP32 pair
            acc[cc][0].A = _f32(xm[cc])
            acc[cc][0].Al = _f32(xm[cc] - np.float64(acc[cc][0].A))
        for s in range(stride):
            n = b * stride + s
            p = phi[n].astype(np.float64)
            x = np.array([x[0] + n01 * x[1] + n02 * x[2], x[1] + n12 * x[2], x[2]]) + np.asarray(svc).T @ p
            zsum += x
            C, G = rows[s]
            if df:
                for cc in range(3):
                    for k in range(3):
                        if C[cc][k] != 0.0:
                            acc[cc][0].add_exact(C[cc][k], phi[n][k])
                            acc[cc][1].add_exact(G[cc][k], phi[n][k])
                    acc[cc][0].renorm()
                    acc[cc][1].renorm()
            else:
                y += C @ p
                v += G @ p
        if df:
            y = np.array([acc[cc][0].value() for cc in range(3)])
            v = np.array([acc[cc][1].value() for cc in range(3)])
        xm, zm = block_end(y, v, zm, float(stride), n01, n02, n12)
        tau = dtau * (b + 1)
        for got, want in ((xm, x), (zm, zsum)):
            g = got[0] + tau * (got[1] + tau * got[2])
            w = want[0] + tau * (want[1] + tau * want[2])
            errs.append(abs(g - w) / (abs(want[0]) + tau * abs(want[1]) + tau * tau * abs(want[2])))
    return max(errs)


@pytest.mark.parametrize("scheme", ["euler", "pc"])
@pytest.mark.parametrize("svc", [SVC_TRI, SVC_GEN], ids=["degree<=k", "general"])
def test_moving_frame_parts_equal_the_fp64_recursion(svc, scheme):
    """In FP64 the block-anchored moving frame's closed forms (M^a, M^-k,
    Q(a)) reproduce the step recursion and its running sums to FP64 rounding:
    1,000 steps of 50 per block, 21 dates, dt = 0.01."""
    assert _moving_frame_errors(svc, 50, 21, 0.01, 0.5, 3, df=False, scheme=scheme) < 1e-13


@pytest.mark.parametrize("svc,seed,scheme", [(SVC_TRI, 0, "euler"), (SVC_TRI, 1, "euler"), (SVC_GEN, 2, "euler"),
                                             (SVC_TRI, 4, "pc")],
                         ids=["degree<=k-0", "degree<=k-1", "general", "pc"])
def test_double_fp32_moving_frame_tracks_the_fp64_recursion(svc, seed, scheme):
    """The kernel's arithmetic: coefficients as FP32 pairs, exact FP32 normals,
    df_acc_w terms packed {y, v}, df_renorm after each part's terms of a step,
    the anchor rounded to an FP32 pair: ~1e-13 of the magnitude of the terms
    at the median date and path (2^-48 of the accumulator per addition over a
    block's ~150 additions; FP64 across blocks), < 7e-13 over 24 seeds."""
    assert _moving_frame_errors(svc, 50, 21, 0.01, 0.5, seed, df=True, scheme=scheme) < 1e-12


# --- mixed precision's response form (hjm_mresp.cu) ---------------------------
@pytest.mark.parametrize("nt,stride,B,c,ns", [(51, 50, 20, 0.02, 8), (51, 50, 24, 0.02, 16)])
def test_mixed_slots_carry_every_counting_date_in_fp32(nt, stride, B, c, ns):
    """The mixed kernel's FP32 sums over its ns slots (the latest dates; the
    host's count, bench.mixed_response_slots) against the direct FP64
    recursion of the remainder: the slotted dates within 4e-6 of their own
    magnitude plus 1e-7 of the largest (FP32 accumulation of FP32-rounded
    terms, one FMA per step: ~sqrt(steps) FP32 roundings, 2e-6 over 1,150
    steps; the running sum's error is then ~1e-10 of the discount exponent,
    far under its own FP32 evaluation), and the dates left without a slot below
    1e-8 |kappa| max|W| per running-sum step (their terms never reach
    2^-30 |kappa|)."""
    import bench

    assert bench.mixed_response_slots(nt, B * stride, stride) == ns
    rng = np.random.default_rng(5)
    W = np.cumsum(rng.normal(size=B * stride)) * 1e-5
    tab, _, kappa = response_table(nt, stride, B, c, 0.5)
    T = tab.reshape(B * stride, ROW, 2).astype(np.float32)
    L = nt - 1
    acc = np.zeros((ns, 2), dtype=np.float32)
    hc = np.zeros(nt)
    hsum = np.zeros(nt)
    w = 0.0
    got, want = {}, {}
    for b in range(1, B):
        for s in range(stride):
            n = b * stride + s
            wf = np.float32(w)
            for r in range(ns):  # every slot every step, as the kernel
                for q in range(2):
                    acc[r, q] = _fma32(T[n, r, q], wf, acc[r, q])
            hn = hc.copy()
            hn[:L] = hc[:L] + c * (hc[1:] - hc[:L])
            hn[L] = hc[L] + c * (hc[L] - hc[L - 1]) + kappa * w
            hc = hn
            hsum += hc
            w = W[n]
        j = b + 1
        want[j] = (hc[j], hsum[j])
        got[j] = (float(acc[B - j, 0]), float(acc[B - j, 1])) if B - j < ns else (0.0, 0.0)
    big = [max(abs(want[j][q]) for j in want) for q in range(2)]
    for j in want:
        for q in range(2):
            if B - j < ns:
                assert abs(got[j][q] - want[j][q]) <= 4e-6 * abs(want[j][q]) + 1e-7 * big[q], (j, q)
            else:
                assert abs(want[j][q]) <= 1e-8 * abs(kappa) * np.max(np.abs(W)) * (j * stride if q else 1), (j, q)
