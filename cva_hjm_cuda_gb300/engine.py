"""Host-side mirror of the reference's exposure interface, over the C ABI.

``calculate_exposure_gpu`` mirrors the reference's
``calculateExposureMultiGPU(expected_exposure, payOff, accrual, spot_rates,
drift, volatilities, scale, num_gpus, simN, dt)`` (simulation_gpu.h:12,14):
same inputs, same 51-point EE output, same print-and-continue behaviour is
left to the C++ drop-in; this Python form raises instead.  ``HJMEngine`` is
the full interface: market and product set-up, FP64 / mixed-precision
valuation with EE, PFE and CVA, external normals, exposures, diagnostics and
the adjoint.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from .market import Market, RunConfig, Swap


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _f64(a) -> np.ndarray:
    return np.ascontiguousarray(a, dtype=np.float64)


@dataclass
class Valuation:
    ee: np.ndarray             # [n_tenor] EE(t_j), zero beyond the last sampled date
    pfe: np.ndarray | None     # [n_tenor] PFE(t_j) or None
    cva: float
    cva_stderr: float
    dcva_dhazard: float
    n_dates: int               # sampled dates + 1


@dataclass
class Sensitivities:
    cva: float
    cva_stderr: float
    dcva_dspot: np.ndarray     # [n_tenor]
    dcva_ddrift: np.ndarray    # [n_tenor]
    dcva_dvolcoef: np.ndarray  # [3, 3]: factor k, power d of T
    dcva_dhazard: float


class HJMEngine:
    """One device context (stream, buffers, market, product)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = C.c_void_p()
        _lib.check(self.lib.hjm_ctx_create(device, C.byref(h)), None)
        self.ctx = h
        self.n_tenor = 0
        self.dtau = 0.5
        self._last_dates = 0
        self._last_paths = 0

    def close(self) -> None:
        if getattr(self, "ctx", None):
            self.lib.hjm_ctx_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, status: int) -> None:
        _lib.check(status, self.ctx)

    # ---------------------------------------------------------------- set-up
    def set_stream(self, cuda_stream: int | None) -> None:
        self._check(self.lib.hjm_ctx_set_stream(self.ctx, C.c_void_p(cuda_stream or 0)))

    def keep_exposures(self, keep: bool = True) -> None:
        self._check(self.lib.hjm_ctx_keep_exposures(self.ctx, 1 if keep else 0))

    def set_memory_limit(self, n_bytes: int) -> None:
        """Cap the device memory of this engine's buffers (0: no cap); a call that
        would grow past it raises HJMError with status HJM_ERR_OUT_OF_MEMORY (4)."""
        self._check(self.lib.hjm_ctx_set_memory_limit(self.ctx, int(n_bytes)))

    def memory_in_use(self) -> int:
        v = C.c_int64(0)
        self._check(self.lib.hjm_ctx_memory_in_use(self.ctx, C.byref(v)))
        return v.value

    def run_mlmc(self, n_paths_per_level, n_steps: int = 1000, dt: float = 0.01, seed: int = 1234,
                 hazard: float = 0.02, recovery: float = 0.4) -> dict:
        """Multi-level Monte Carlo EE / CVA: level l uses dt / 2^l on
        n_paths_per_level[l] paths (hjm_run_mlmc).  Returns the summed EE, CVA
        and standard error, and per level the CVA difference, its standard
        error, the device ms and the path count."""
        n = np.ascontiguousarray(n_paths_per_level, dtype=np.int64)
        nt = self.n_tenor
        ee, cva, lev = np.zeros(nt), np.zeros(3), np.zeros(4 * n.size)
        self._check(self.lib.hjm_run_mlmc(self.ctx, n.size, n.ctypes.data_as(C.POINTER(C.c_int64)), n_steps, dt,
                                          seed, hazard, recovery, _dptr(ee), _dptr(cva), _dptr(lev)))
        lev = lev.reshape(n.size, 4)
        return {"ee": ee, "cva": cva[0], "cva_stderr": cva[1], "dcva_dhazard": cva[2],
                "levels": [{"cva_diff": r[0], "stderr": r[1], "ms": r[2], "n_paths": int(r[3])} for r in lev]}

    def set_scheme(self, scheme: str = "euler") -> None:
        """Time scheme of the Musiela SDE: "euler" (the reference's) or
        "predictor_corrector"."""
        self._check(self.lib.hjm_ctx_set_scheme(self.ctx, {"euler": 0, "predictor_corrector": 1}[scheme]))

    def set_remainder_form(self, form: str = "auto") -> None:
        """Transport form of the remainder: "convect" (the remainder, or with a
        table of any shape the whole stochastic curve, over the live tenors
        every step), "response" (impulse-response sums at the sampled tenors:
        FP64 valuations in double-FP32, in windows of dates; mixed precision
        and its adjoint without checkpoints in FP32 where the dates the
        remainder reaches fit 16 slots) or "auto" (the response form where it
        applies)."""
        self._check(self.lib.hjm_ctx_set_remainder_form(self.ctx, {"auto": 0, "convect": 1, "response": 2}[form]))

    def remainder_form(self) -> str:
        """The remainder form of the last valuation enqueued: "none" (table
        step), "convect" or "response"."""
        form = C.c_int32(0)
        self._check(self.lib.hjm_ctx_remainder_form(self.ctx, C.byref(form)))
        return ("none", "convect", "response")[form.value]

    def write_report(self, path, fmt: str = "json") -> None:
        """The last valuation (or adjoint run) with its inputs, as JSON or CSV."""
        code = {"json": 0, "csv": 1}[fmt]
        self._check(self.lib.hjm_write_report(self.ctx, str(path).encode(), code))

    def vol_decomposition(self, enable: bool | None = None) -> bool:
        """Allow (True) or forbid (False) the polynomial volatility decomposition;
        returns whether the current market runs it."""
        if enable is not None:
            self._check(self.lib.hjm_ctx_set_vol_decomposition(self.ctx, 1 if enable else 0))
        return self.vol_form() != "table"

    def vol_form(self) -> str:
        """The step the current market runs: "table", "poly" (quadratic factors),
        "poly_tri" (factor k of degree <= k) or "cubic_resid" (cubic factors up to a
        residual table: the FP64 Euler valuations; other modes run the table step)."""
        active = C.c_int32(0)
        self._check(self.lib.hjm_ctx_vol_decomposition(self.ctx, C.byref(active)))
        return ("table", "poly", "poly_tri", "cubic_resid")[active.value]

    def set_market(self, market: Market, drift: bool = True) -> None:
        spot, vol = _f64(market.spot), _f64(market.vol).ravel()
        d = _f64(market.drift) if drift else None
        self._check(self.lib.hjm_set_market(self.ctx, market.n_tenor, market.dtau, _dptr(spot), _dptr(vol), 3,
                                            _dptr(d) if d is not None else None))
        self.n_tenor, self.dtau = market.n_tenor, market.dtau

    def set_market_poly(self, n_tenor: int, dtau: float, spot, vol_coeffs) -> None:
        spot = _f64(spot)
        coef = _f64(vol_coeffs).reshape(9)
        self._check(self.lib.hjm_set_market_poly(self.ctx, n_tenor, dtau, _dptr(spot), _dptr(coef)))
        self.n_tenor, self.dtau = n_tenor, dtau

    def set_swap(self, swap: Swap) -> None:
        acc = _f64(swap.accrual)
        self._check(self.lib.hjm_set_swap(self.ctx, swap.notional, swap.strike, _dptr(acc), 1 if swap.payer else 0))

    def set_netting_set(self, netting=None, notional=None, fixed_rate=None, n_periods=None, payer=None) -> None:
        if netting is not None:
            notional, fixed_rate, n_periods, payer = (netting.notional, netting.fixed_rate, netting.n_periods,
                                                      netting.payer)
        n = len(notional)
        notional, fixed_rate = _f64(notional), _f64(fixed_rate)
        n_periods = np.ascontiguousarray(n_periods, dtype=np.int32)
        payer = np.ascontiguousarray(payer, dtype=np.int32)
        ip = C.POINTER(C.c_int32)
        self._check(self.lib.hjm_set_netting_set(self.ctx, n, _dptr(notional), _dptr(fixed_rate),
                                                 n_periods.ctypes.data_as(ip), payer.ctypes.data_as(ip)))

    # ------------------------------------------------------------- valuation
    def run(self, cfg: RunConfig, precision: str = "fp64", pfe: bool = True) -> Valuation:
        nt = self.n_tenor
        ee, pf, cva = np.zeros(nt), np.zeros(nt), np.zeros(3)
        self._check(self.lib.hjm_run(self.ctx, cfg.n_paths, cfg.n_steps, cfg.dt, cfg.seed, cfg.path_offset,
                                     _lib.PRECISION[precision], cfg.hazard, cfg.recovery, cfg.pfe_quantile,
                                     _dptr(ee), _dptr(pf) if pfe else None, _dptr(cva)))
        self._last_paths = cfg.n_paths
        self._last_dates = cfg.n_steps // int(round(self.dtau / cfg.dt)) + 1
        return Valuation(ee, pf if pfe else None, float(cva[0]), float(cva[1]), float(cva[2]), self._last_dates)

    def enqueue(self, cfg: RunConfig, precision: str = "fp64", pfe: bool = True) -> None:
        self._check(self.lib.hjm_enqueue(self.ctx, cfg.n_paths, cfg.n_steps, cfg.dt, cfg.seed, cfg.path_offset,
                                         _lib.PRECISION[precision], cfg.hazard, cfg.recovery,
                                         cfg.pfe_quantile if pfe else 0.0))
        self._last_paths = cfg.n_paths
        self._last_dates = cfg.n_steps // int(round(self.dtau / cfg.dt)) + 1

    def fetch(self, pfe: bool = True) -> Valuation:
        nt = self.n_tenor
        ee, pf, cva = np.zeros(nt), np.zeros(nt), np.zeros(3)
        self._check(self.lib.hjm_fetch_results(self.ctx, _dptr(ee), _dptr(pf), _dptr(cva)))
        return Valuation(ee, pf if pfe else None, float(cva[0]), float(cva[1]), float(cva[2]), self._last_dates)

    def run_with_normals(self, normals: np.ndarray, n_steps: int, dt: float, precision: str = "fp64",
                         hazard: float = 0.02, recovery: float = 0.4, pfe_quantile: float = 0.975,
                         pfe: bool = True) -> Valuation:
        normals = _f64(normals)
        n_paths = normals.shape[0]
        if normals.shape != (n_paths, n_steps, 3):
            raise ValueError(f"normals must be [n_paths][{n_steps}][3], got {normals.shape}")
        nt = self.n_tenor
        ee, pf, cva = np.zeros(nt), np.zeros(nt), np.zeros(3)
        self._check(self.lib.hjm_run_with_normals(self.ctx, n_paths, n_steps, dt, _dptr(normals),
                                                  _lib.PRECISION[precision], hazard, recovery, pfe_quantile,
                                                  _dptr(ee), _dptr(pf) if pfe else None, _dptr(cva)))
        self._last_paths = n_paths
        self._last_dates = n_steps // int(round(self.dtau / dt)) + 1
        return Valuation(ee, pf if pfe else None, float(cva[0]), float(cva[1]), float(cva[2]), self._last_dates)

    def exposures(self) -> np.ndarray:
        """Per-path exposures of the last valuation, [n_dates][n_paths]."""
        out = np.zeros((self._last_dates, self._last_paths))
        self._check(self.lib.hjm_get_exposures(self.ctx, _dptr(out), out.size))
        return out

    def exposure_paths(self, path_begin: int, n: int) -> np.ndarray:
        """Per-path exposures of the paths [path_begin, path_begin + n) of the
        last valuation, [n_dates][n]: only that slice leaves the device."""
        out = np.zeros((self._last_dates, n))
        self._check(self.lib.hjm_get_exposure_paths(self.ctx, path_begin, n, _dptr(out)))
        return out

    # ---------------------------------------------------------- sensitivities
    def run_adjoint(self, cfg: RunConfig, checkpoint_every: int = 32) -> Sensitivities:
        nt = self.n_tenor
        cva = np.zeros(3)
        dspot, ddrift, dcoef = np.zeros(nt), np.zeros(nt), np.zeros(9)
        self._check(self.lib.hjm_run_adjoint(self.ctx, cfg.n_paths, cfg.n_steps, cfg.dt, cfg.seed, cfg.path_offset,
                                             cfg.hazard, cfg.recovery, checkpoint_every, _dptr(cva), _dptr(dspot),
                                             _dptr(ddrift), _dptr(dcoef)))
        return Sensitivities(float(cva[0]), float(cva[1]), dspot, ddrift, dcoef.reshape(3, 3), float(cva[2]))

    # ------------------------------------------------------------ diagnostics
    def dump_normals(self, n_paths: int, n_steps: int, seed: int, path_offset: int = 0) -> np.ndarray:
        out = np.zeros((n_paths, n_steps, 3))
        self._check(self.lib.hjm_dump_normals(self.ctx, n_paths, path_offset, n_steps, seed, _dptr(out)))
        return out

    def philox_words(self, n_paths: int, step: int, seed: int, path_offset: int = 0) -> np.ndarray:
        out = np.zeros((n_paths, 4), dtype=np.uint32)
        self._check(self.lib.hjm_philox_words(self.ctx, n_paths, path_offset, step, seed,
                                              out.ctypes.data_as(C.POINTER(C.c_uint32))))
        return out

    def timings(self) -> dict:
        ms = np.zeros(4)
        self._check(self.lib.hjm_last_timings(self.ctx, _dptr(ms)))
        return {"path_ms": ms[0], "reduce_ms": ms[1], "pfe_ms": ms[2], "total_ms": ms[3]}

    def timing_history(self, n: int) -> np.ndarray:
        """[n][4] device ms of the last n valuations: path kernel, reductions, PFE, total."""
        ms = np.zeros((n, 4))
        self._check(self.lib.hjm_timing_history(self.ctx, n, _dptr(ms)))
        return ms

    def stats(self) -> dict:
        v = np.zeros(3, dtype=np.int64)
        self._check(self.lib.hjm_last_stats(self.ctx, v.ctypes.data_as(C.POINTER(C.c_int64))))
        return {"kernels": int(v[0]), "h2d_bytes": int(v[1]), "d2h_bytes": int(v[2])}

    def fma_peak_tflops(self, precision: str = "fp64") -> float:
        v = C.c_double(0.0)
        self._check(self.lib.hjm_measure_fma_peak(self.ctx, _lib.PRECISION[precision], C.byref(v)))
        return v.value


@dataclass
class Calibration:
    vol: np.ndarray        # [3][n_tenor] factor volatilities sqrt(lambda_k) e_k
    eigval: np.ndarray     # [3] annualised eigenvalues, descending
    vol_coeffs: np.ndarray # [3][3] polynomial fit of factor k, degree min(k, 2)
    explained: float       # share of the total variance the three factors carry

    def market(self, spot, dtau: float = 0.5, poly: bool = True) -> Market:
        """A Market on the calibrated factors: the polynomial fit (poly) or the raw table."""
        spot = np.asarray(spot, dtype=np.float64)
        if poly:
            return Market(n_tenor=spot.size, dtau=dtau, spot=spot, vol_coeffs=self.vol_coeffs.copy())
        return Market(n_tenor=spot.size, dtau=dtau, spot=spot, vol=self.vol.copy())


def mlmc_allocation(level_var, level_cost, target_stderr: float, min_paths: int = 1024) -> np.ndarray:
    """Paths per level minimising the cost for a target standard error
    (Giles 2008): N_l = ceil(sqrt(V_l / C_l) * sum_k sqrt(V_k C_k) / eps^2),
    with V_l the per-path variance and C_l the per-path cost of level l; at
    least min_paths per level so that every level's variance is estimated."""
    v = np.asarray(level_var, dtype=np.float64)
    c = np.asarray(level_cost, dtype=np.float64)
    if np.any(v < 0) or np.any(c <= 0) or target_stderr <= 0:
        raise ValueError("variances >= 0, costs > 0 and a positive target are required")
    n = np.sqrt(v / c) * np.sum(np.sqrt(v * c)) / target_stderr**2
    return np.maximum(np.ceil(n), min_paths).astype(np.int64)


def calibrate_pca(curves, dtau: float = 0.5, obs_per_year: float = 252.0) -> Calibration:
    """Volatility factors from historical forward curves [n_obs][n_tenor]
    (hjm_calibrate_pca: principal components of the annualised covariance of
    the curve changes, then a polynomial fit of each factor)."""
    curves = _f64(curves)
    if curves.ndim != 2:
        raise ValueError("curves must be [n_obs][n_tenor]")
    n_obs, nt = curves.shape
    lib = _lib.load()
    vol, eig, coef, expl = np.zeros(3 * nt), np.zeros(3), np.zeros(9), C.c_double(0.0)
    st = lib.hjm_calibrate_pca(_dptr(curves), n_obs, nt, dtau, obs_per_year, 3, _dptr(vol), _dptr(eig), _dptr(coef),
                               C.byref(expl))
    _lib.check(st)
    return Calibration(vol.reshape(3, nt), eig, coef.reshape(3, 3), expl.value)


def calculate_exposure_gpu(expected_exposure: np.ndarray, notional: float, K: float, expiry: float, dtau: float,
                           accrual, spot_rates, drift, volatilities, scale: float, num_gpus: int, simN: int,
                           dt: float) -> None:
    """The reference's calculateExposureMultiGPU (double overload) through the
    C++ drop-in of libhjmcva.so; writes the 51-point EE into expected_exposure."""
    lib = _lib.load()
    if expected_exposure.dtype != np.float64 or expected_exposure.size < 51:
        raise ValueError("expected_exposure must be a float64 array of 51 values")
    a, s, d, v = (_f64(x) for x in (accrual, spot_rates, drift, volatilities))
    lib.hjm_dropin_calculate_exposure_fp64(_dptr(expected_exposure), notional, K, expiry, dtau, _dptr(a), _dptr(s),
                                           _dptr(d), _dptr(v), num_gpus, simN, dt)


def calculate_exposure_gpu_fp32(expected_exposure: np.ndarray, notional: float, K: float, expiry: float, dtau: float,
                                accrual, spot_rates, drift, volatilities, scale: float, num_gpus: int, simN: int,
                                dt: float) -> None:
    """The float overload of calculateExposureMultiGPU (simulation_gpu.h:14, the
    library's mixed precision) through the C++ drop-in; float32 arrays in, the
    51-point EE written into expected_exposure (float32)."""
    lib = _lib.load()
    if expected_exposure.dtype != np.float32 or expected_exposure.size < 51:
        raise ValueError("expected_exposure must be a float32 array of 51 values")
    a, s, d, v = (np.ascontiguousarray(x, dtype=np.float32) for x in (accrual, spot_rates, drift, volatilities))
    fp = lambda x: x.ctypes.data_as(C.POINTER(C.c_float))  # noqa: E731
    lib.hjm_dropin_calculate_exposure_fp32(fp(expected_exposure), notional, K, expiry, dtau, fp(a), fp(s), fp(d),
                                           fp(v), num_gpus, simN, dt)
