"""CPU checks of the generalised Euler response form (hjm_eresp.cu), in numpy.

* The cubic decomposition of a volatility table up to a residual: the
  reference driver's own PCA table (simulation_gpu_testing.cpp:47-63, stored
  in the driver's golden fixture) fits factor 1 by a constant and factors 2
  and 3 by cubics in t = T - T_L, with residuals of the table's 9-decimal
  rounding (about 1e-7 of each factor's scale); a quadratic leaves 0.5 of it.
* The algebra: the stochastic curve evolved by the Euler step on the whole
  table (h <- A h + sqrt(dt) sigma phi, the reference's step with zero drift)
  equals, at every sampled date's tenor and for its running sum, the cubic
  parts x <- M x + B phi (basis centred at tau0: T_L, or the middle of the
  sampled tenors) plus the remainder's impulse-response sums kappa G_j w +
  R_jk phi, w = x_2 + 3 (T_L - tau0) x_3 read before the step, to FP64
  rounding.
* The moving frame with four parts: y += C(s) phi, v += G(s) phi within a
  block, x = M^a y and sum = Q(a) y - v at its end, and W before step s =
  y_W + s n23 y_X, against the direct recursion of the parts.
* The windows: every date is priced by exactly one window, every window holds
  at most 24 dates that can be active (from the first date the remainder
  reaches, eresp_first_active_date, on), the latest window is run first.
* The active prefix of the response table (eresp_active_kernel): the terms it
  skips sum, per date, to less than 32 x 2^-53 |kappa| per unit |W|, and the
  sums over it equal the convected remainder.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import load_golden

TOL = 2.0 ** -20
SLOTS = 24


def fit_cubic_resid(vol, nt, dtau):
    """Restatement of the library's fit: per factor the lowest degree <= 3 whose
    least-squares residual is at most 2^-20 of the factor's scale, in t = T - T_L."""
    TL = dtau * (nt - 1)
    T = dtau * np.arange(nt)
    u = (T - TL) / TL
    coef, degs, resid = np.zeros((3, 4)), [], np.zeros((3, nt))
    for k in range(3):
        v = vol[k]
        scale = np.max(np.abs(v))
        for d in range(4):
            V = np.vander(u, d + 1, increasing=True)
            b, *_ = np.linalg.lstsq(V, v, rcond=None)
            a = b / TL ** np.arange(d + 1)
            pv = np.polyval(a[::-1], T - TL)
            if np.max(np.abs(v - pv)) <= TOL * scale:
                coef[k, : d + 1] = a
                degs.append(d)
                resid[k] = v - pv
                break
        else:
            return None
    return coef, degs, resid


def reference_table():
    g = load_golden("ref_driver_own_market.json")
    return np.array(g["vol"]).reshape(3, 51)


def test_reference_table_is_cubic_to_its_rounding():
    vol = reference_table()
    fit = fit_cubic_resid(vol, 51, 0.5)
    assert fit is not None
    coef, degs, resid = fit
    assert degs == [0, 3, 3]
    for k in range(3):
        rel = np.max(np.abs(resid[k])) / np.max(np.abs(vol[k]))
        assert rel < 2e-7, (k, rel)
    # a quadratic does not fit factors 2 and 3
    T = 0.5 * np.arange(51)
    for k in (1, 2):
        q = np.polyfit(T, vol[k], 2)
        assert np.max(np.abs(vol[k] - np.polyval(q, T))) > 0.3 * np.max(np.abs(vol[k]))


def upwind(v, c):
    L = v.size - 1
    w = v.copy()
    w[:L] = v[:L] + c * (v[1:] - v[:L])
    w[L] = v[L] + c * (v[L] - v[L - 1])
    return w


def parts_matrix(c, dtau):
    """N[i][d] = c C(d, i) dtau^(d - i): the upwind step on the monomials t^d."""
    from math import comb

    N = np.zeros((4, 4))
    for d in range(4):
        for i in range(d):
            N[i, d] = c * comb(d, i) * dtau ** (d - i)
    return N


def _direct(vol, nt, stride, B, dt, phi):
    """The Euler step on the whole table (stochastic part only): h and its running
    sum at each date's tenor at the date's sampling step."""
    c = dt / 0.5
    h = np.zeros(nt)
    acc = np.zeros(nt)
    hs, accs = np.zeros(B + 1), np.zeros(B + 1)
    for n in range(stride, B * stride):
        h = upwind(h, c) + np.sqrt(dt) * (vol.T @ phi[n])
        acc += h
        if (n + 1) % stride == 0:
            j = (n + 1) // stride
            hs[j], accs[j] = h[j], acc[j]
    return hs, accs


def _shift(coef, d):
    """Coefficients of (T - T_L)^e re-expanded in powers of (T - T_L - d)."""
    from math import comb

    out = np.zeros_like(coef)
    for k in range(coef.shape[0]):
        for dd in range(4):
            out[k, dd] = sum(comb(e, dd) * coef[k, e] * d ** (e - dd) for e in range(dd, 4))
    return out


def _decomposed(coef, resid, nt, stride, B, dt, phi, tau0=None):
    """Cubic parts + the remainder's response sums, in FP64 (the kernel's algebra)."""
    dtau = 0.5
    c = dt / dtau
    L = nt - 1
    TL = dtau * L
    tau0 = TL if tau0 is None else tau0
    kappa = -2.0 * c * dtau * dtau
    N = parts_matrix(c, dtau)
    M = np.eye(4) + N
    Bm = np.sqrt(dt) * _shift(coef, tau0 - TL).T  # [part][factor], basis T - tau0
    r = np.sqrt(dt) * resid  # [factor][tenor]
    # responses G_j(m), R_jk(m) and running sums by repeated upwind steps
    Mmax = (B - 1) * stride
    G = np.zeros((Mmax, nt))
    R = np.zeros((Mmax, 3, nt))
    g = np.zeros(nt)
    g[L] = 1.0
    rr = r.copy()
    for m in range(Mmax):
        G[m], R[m] = g, rr
        g = upwind(g, c)
        rr = np.array([upwind(rr[k], c) for k in range(3)])
    CG, CR = np.cumsum(G, axis=0), np.cumsum(R, axis=0)
    x = np.zeros(4)
    X = np.zeros(4)
    hc, hcs = np.zeros(B + 1), np.zeros(B + 1)
    hs, accs = np.zeros(B + 1), np.zeros(B + 1)
    for n in range(stride, B * stride):
        W = x[2] + 3.0 * (TL - tau0) * x[3]  # the source, before the step
        for j in range(2, B + 1):
            lag = j * stride - 1 - n
            if lag < 0:
                continue
            hc[j] += kappa * G[lag, j] * W + R[lag, :, j] @ phi[n]
            hcs[j] += kappa * CG[lag, j] * W + CR[lag, :, j] @ phi[n]
        x = M @ x + Bm @ phi[n]
        X += x
        if (n + 1) % stride == 0:
            j = (n + 1) // stride
            t = dtau * j - tau0
            p = t ** np.arange(4)
            hs[j], accs[j] = x @ p + hc[j], X @ p + hcs[j]
    return hs, accs


@pytest.mark.parametrize("centre", ["last-tenor", "middle-of-dates"])
@pytest.mark.parametrize("stride,B,seed", [(50, 20, 1), (25, 12, 2), (10, 30, 3)])
def test_cubic_parts_plus_responses_equal_the_euler_step(stride, B, seed, centre):
    vol = reference_table()
    coef, degs, resid = fit_cubic_resid(vol, 51, 0.5)
    dt = 0.5 / stride
    phi = np.random.default_rng(seed).standard_normal((B * stride, 3))
    tau0 = None if centre == "last-tenor" else 0.25 * (1 + B)
    hd, ad = _direct(vol, 51, stride, B, dt, phi)
    hr, ar = _decomposed(coef, resid, 51, stride, B, dt, phi, tau0)
    scale_h, scale_a = np.max(np.abs(hd)), np.max(np.abs(ad))
    assert np.max(np.abs(hd[2:] - hr[2:])) < 1e-12 * scale_h
    assert np.max(np.abs(ad[2:] - ar[2:])) < 1e-12 * scale_a
    # without the residual responses the difference is of the residual's size
    hr0, _ = _decomposed(coef, np.zeros_like(resid), 51, stride, B, dt, phi)
    assert np.max(np.abs(hd[2:] - hr0[2:])) > 1e-9 * scale_h


def _binom(a, i):
    out = 1.0
    for j in range(i):
        out = out * (a - j) / (j + 1)
    return out


def _poly_n(N, c0, c1, c2, c3):
    return c0 * np.eye(4) + c1 * N + c2 * N @ N + c3 * N @ N @ N


@pytest.mark.parametrize("stride", [50, 7])
def test_four_part_moving_frame_equals_the_parts_recursion(stride):
    dtau, dt = 0.5, 0.5 / stride
    c = dt / dtau
    N = parts_matrix(c, dtau)
    M = np.eye(4) + N
    rng = np.random.default_rng(11)
    Bm = rng.normal(size=(4, 3)) * 1e-3
    # the closed forms the kernels use
    for a in (1, 3, stride):
        Ma = _poly_n(N, 1.0, _binom(a, 1), _binom(a, 2), _binom(a, 3))
        assert np.allclose(Ma, np.linalg.matrix_power(M, a), rtol=1e-14, atol=1e-17)
        Qa = _poly_n(N, a, _binom(a + 1, 2), _binom(a + 1, 3), _binom(a + 1, 4))
        assert np.allclose(Qa, sum(np.linalg.matrix_power(M, e) for e in range(1, a + 1)), rtol=1e-13, atol=1e-17)
        k = a
        Mk = _poly_n(N, 1.0, -k, 0.5 * k * (k + 1), -(k + 2) * (k + 1) * k / 6.0)
        assert np.allclose(Mk, np.linalg.matrix_power(np.linalg.inv(M), k), rtol=1e-13, atol=1e-17)
    # one block in the frame against the direct recursion, from a nonzero start
    x0 = rng.normal(size=4) * 1e-2
    phi = rng.standard_normal((stride, 3))
    x, xs, Ws = x0.copy(), np.zeros(4), []
    for s in range(stride):
        Ws.append(x[2])
        x = M @ x + Bm @ phi[s]
        xs += x
    y, v = x0.copy(), np.zeros(4)
    n23 = N[2, 3]
    for s in range(stride):
        assert abs((y[2] + s * n23 * y[3]) - Ws[s]) < 1e-15 * max(1.0, abs(Ws[s]))
        k = s + 1
        C = _poly_n(N, 1.0, -k, 0.5 * k * (k + 1), -(k + 2) * (k + 1) * k / 6.0) @ Bm
        Q = _poly_n(N, s, _binom(s + 1, 2), _binom(s + 1, 3), _binom(s + 1, 4))
        y = y + C @ phi[s]
        v = v + (Q @ C) @ phi[s]
    a = stride
    Ma = _poly_n(N, 1.0, _binom(a, 1), _binom(a, 2), _binom(a, 3))
    Qa = _poly_n(N, a, _binom(a + 1, 2), _binom(a + 1, 3), _binom(a + 1, 4))
    assert np.allclose(Ma @ y, x, rtol=1e-12, atol=1e-16)
    assert np.allclose(Qa @ y - v, xs, rtol=1e-12, atol=1e-15)


def windows(B, first=2, dates=SLOTS):
    """Restatement of eresp_windows: latest first, (lo, hi, ns); dates before
    first never need a slot; ``dates`` per window (24, or 16 with a residual
    table, eresp_window_dates, and for the volatility-table response form)."""
    f = max(first, 2)
    out, h = [], B
    while h >= 1:
        lo = 1
        if h - f + 1 > dates:
            lo = h - dates + 1
            if lo <= 2:
                lo = 1
        act = max(h - max(lo, f) + 1, 0)
        ns = 12 if act <= 12 else (16 if act <= 16 else (20 if act <= 20 else 24))
        out.append((lo, h, ns))
        h = lo - 1
    return out


@pytest.mark.parametrize("first", [2, 10, 13])
@pytest.mark.parametrize("B", list(range(1, 61)))
def test_windows_partition_the_dates(B, first):
    w16 = windows(B, first, 16)
    assert sorted(d for lo, hi, _ in w16 for d in range(lo, hi + 1)) == list(range(1, B + 1))
    assert all(hi - max(lo, first, 2) + 1 <= 16 for lo, hi, _ in w16)
    w = windows(B, first)
    dates = sorted(d for lo, hi, _ in w for d in range(lo, hi + 1))
    assert dates == list(range(1, B + 1))
    for lo, hi, ns in w:
        active = max(hi - max(lo, first, 2) + 1, 0)
        assert active <= ns <= SLOTS
        assert hi - max(lo, 2) + 1 <= SLOTS or lo == 1
    assert w[0][1] == B and w[-1][0] == 1
    assert [hi for _, hi, _ in w] == sorted((hi for _, hi, _ in w), reverse=True)
    if B <= 25 or B - max(first, 2) + 1 <= SLOTS:
        assert [(lo, hi) for lo, hi, _ in w] == [(1, B)]
    if first == 2:
        # every date with a slot: the windows of 24 slotted dates
        h = B
        for lo, hi, _ in w:
            assert hi == h and lo == (1 if h - 23 <= 2 else h - 23)
            h = lo - 1


# --- the active prefixes of the Euler response table (eresp_active_kernel) ---
def eresp_table(nt, stride, B, c, dtau=0.5):
    """kappa G_j(lag) and kappa CG_j(lag) per (row n = b stride + s, global slot
    B - j), lag = j stride - 1 - n, as eresp_table_kernel writes them (FP64)."""
    L = nt - 1
    kappa = -2.0 * c * dtau * dtau
    rows = B * stride
    tab = np.zeros((rows, B + 1, 2))
    v = np.zeros(nt)
    v[L] = 1.0
    cum = np.zeros(nt)
    for m in range((B - 1) * stride):
        cum = cum + v
        for t in range(2, B + 1):
            n = t * stride - 1 - m
            if n >= stride:
                tab[n, B - t] = (kappa * v[t], kappa * cum[t])
        v = upwind(v, c)
    return tab, kappa


def eresp_prefix(tab, kappa, B, stride):
    """As eresp_active_kernel without a residual: per row, the slots up to the
    last whose FP32 kappa G reaches 2^-53 |kappa| or kappa CG reaches 2^-53
    |kappa| times the date's sampling step."""
    a = np.abs(tab.astype(np.float32))
    tg = np.float32(abs(kappa)) * np.float32(2.0 ** -53)
    dates = np.maximum(B - np.arange(tab.shape[1]), 1)
    tcg = (tg * (dates * stride).astype(np.float32)).astype(np.float32)
    sig = ((a[:, :, 0] != 0) & (a[:, :, 0] >= tg)) | ((a[:, :, 1] != 0) & (a[:, :, 1] >= tcg[None, :]))
    return np.where(sig.any(axis=1), tab.shape[1] - np.argmax(sig[:, ::-1], axis=1), 0)


ERESP_SHAPES = [(51, 50, 20), (51, 50, 24), (61, 50, 24), (51, 25, 20), (51, 100, 10), (51, 10, 5)]


@pytest.mark.parametrize("nt,stride,B", ERESP_SHAPES)
def test_eresp_prefix_drops_only_terms_below_the_unit_roundoff(nt, stride, B):
    """The prefix skips, per date, terms that sum to less than 32 x 2^-53 |kappa|
    per unit |W| (and per sampling step for the running sum), and at the 10y
    shape a quarter of the terms the nonzero prefix would keep."""
    c = (0.5 / stride) / 0.5
    tab, kappa = eresp_table(nt, stride, B, c)
    pre = eresp_prefix(tab, kappa, B, stride)
    nz = np.where((tab != 0).any(axis=2).any(axis=1),
                  tab.shape[1] - np.argmax((tab != 0).any(axis=2)[:, ::-1], axis=1), 0)
    assert np.all(pre <= nz)
    for t in range(2, B + 1):
        r = B - t
        rows = np.arange(stride, t * stride)
        dropped = rows[pre[rows] <= r]
        dg = np.abs(tab[dropped, r, 0]).sum()
        dcg = np.abs(tab[dropped, r, 1]).sum()
        assert dg <= 32 * 2.0 ** -53 * abs(kappa), (t, dg)
        assert dcg <= 32 * 2.0 ** -53 * abs(kappa) * t * stride, (t, dcg)
    if (nt, stride, B) == (51, 50, 20):
        groups = lambda p: 4 * ((p[stride:] + 3) // 4)
        assert groups(pre).mean() < 0.8 * groups(nz).mean()


@pytest.mark.parametrize("nt,stride,B", ERESP_SHAPES[:4])
def test_eresp_prefix_sums_equal_the_convected_remainder(nt, stride, B):
    """The response sums over the prefix against hc <- A hc + kappa W e_L,
    to 1e-12 of each sum plus the dropped terms' bound."""
    c = (0.5 / stride) / 0.5
    tab, kappa = eresp_table(nt, stride, B, c)
    pre = eresp_prefix(tab, kappa, B, stride)
    L = nt - 1
    W = np.cumsum(np.random.default_rng(3).normal(size=B * stride)) * 1e-5
    acc = np.zeros((B + 1, 2))
    hc, hs = np.zeros(nt), np.zeros(nt)
    for n in range(stride, B * stride):
        w = W[n - 1]
        acc[: pre[n]] += tab[n, : pre[n]] * w
        hc = upwind(hc, c)
        hc[L] += kappa * w
        hs += hc
        if (n + 1) % stride == 0:
            j = (n + 1) // stride
            if j >= 2:
                floor = 32 * 2.0 ** -53 * abs(kappa) * np.abs(W).max()
                assert abs(acc[B - j, 0] - hc[j]) <= 1e-12 * abs(hc[j]) + floor
                assert abs(acc[B - j, 1] - hs[j]) <= 1e-12 * abs(hs[j]) + floor * j * stride


def first_active_date(nt, stride, B):
    """Restatement of eresp_first_active_date (no residual): the earliest date
    whose kappa G or kappa CG reaches half the device's threshold at some lag
    its entries hold."""
    c = (0.5 / stride) / 0.5
    L = nt - 1
    v = np.zeros(nt)
    v[L] = 1.0
    cum = np.zeros(nt)
    sig = np.zeros(B + 1, bool)
    for m in range((B - 1) * stride):
        cum = cum + v
        for t in range(2, B + 1):
            if m <= (t - 1) * stride - 1 and (abs(v[t]) >= 2.0 ** -54 or abs(cum[t]) >= 2.0 ** -54 * t * stride):
                sig[t] = True
        v = upwind(v, c)
    hits = np.nonzero(sig)[0]
    return int(hits[0]) if hits.size else B + 1


@pytest.mark.parametrize("nt,stride,B", ERESP_SHAPES + [(51, 50, 30), (61, 50, 36)])
def test_first_active_date_bounds_the_device_prefix(nt, stride, B):
    """No row's active prefix reaches a date before the first active date, so
    the windows' slots from it on (eresp_windows) hold every active term; at
    the 10y shape the remainder never reaches dates 2 to 9."""
    c = (0.5 / stride) / 0.5
    tab, kappa = eresp_table(nt, stride, B, c)
    pre = eresp_prefix(tab, kappa, B, stride)
    f = first_active_date(nt, stride, B)
    assert pre.max() <= max(B - f + 1, 0)
    if (nt, stride, B) == (51, 50, 20):
        assert f == 10 and pre.max() == 11
        assert windows(B, f) == [(1, 20, 12)]
    if (nt, stride, B) == (51, 50, 30):
        assert [(lo, hi) for lo, hi, _ in windows(B, f)] == [(1, 30)]
