"""Generate the golden vectors in this folder from the reference itself.

Run from the repository root, where the reference tree is present (its path in
HJM_REFERENCE_DIR, default /root/reference):

    python tests/golden/make_golden.py

It compiles the reference's own CPU path (oracle/Makefile, target ``ref``),
reproduces the reference's own normal draws (cuRAND host XORWOW, seed 1234,
simulation_cpu.h:83-90 and :399) and writes:

* ``ref_driver_25y.json`` -- the EE profile returned by the reference's whole,
  unmodified ``calculateExposureCPU<double>`` (simulation_cpu.h:350) for a 25y
  payer swap (every block of the 51-tenor grid is sampled, so the reference
  reads no uninitialised numeraire);
* ``ref_blocks_10y.json`` -- the reference's per-path functions driven over a
  10y swap (1,000 steps, 20 sampled dates) with zeroed numeraires: EE and the
  exposure rows of the first paths;
* ``ref_driver_own_market.json`` -- the reference driver's own workload
  (simulation_gpu_testing.cpp): its BoE spot curve (:36-41), PCA volatility
  table (:47-63), hard-coded drift table (:66-71) and irregular 30/360
  accruals (:117-123), the swap N = 10, K = 6.7%, 25y, dtau 0.5
  (:147-148, :215), dt = 0.01, 5,000 paths -- the EE of the whole, unmodified
  calculateExposureCPU<double> (the driver's ``-cpu -scenarios 5000`` run)
  and the exposure rows of the first paths from the reference's per-path
  functions.  The arrays are read from the driver's source text.

The first two use the synthetic market of the configured workloads
(Nelson-Siegel curve, polynomial volatility factors, trapezoid drift).  Every
input is stored in the fixtures verbatim, so tests do not depend on
regenerating them.  Before writing, the oracle restatement is checked against
the reference on the same normals.
"""
from __future__ import annotations

import json
import os
import re
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "tests"))

import oracle_lib as O  # noqa: E402
from cva_hjm_cuda_gb300.market import Market, Swap  # noqa: E402

REFERENCE = Path(os.environ.get("HJM_REFERENCE_DIR", "/root/reference"))


def driver_array(src: str, name: str) -> np.ndarray:
    """A numeric array initialiser of the reference driver, by variable name."""
    m = re.search(r"(?:real|double|float)\s+" + name + r"\[\d*\]\s*=\s*\{(.*?)\};", src, re.S)
    if m is None:
        m = re.search(r"std::vector<\w+>\s+" + name + r"\s*=\s*\{(.*?)\};", src, re.S)
    if m is None:
        raise KeyError(name)
    return np.array([float(x) for x in m.group(1).replace("\n", " ").split(",") if x.strip()])


def market_inputs(n_periods: int):
    mk = Market(n_tenor=51, dtau=0.5)
    mk.drift = O.trapezoid_drift(mk.vol, mk.dtau)
    sw = Swap(notional=1.0e6, strike=0.025, n_periods=n_periods, n_tenor=51, dtau=0.5)
    return mk, sw


def dump(path: Path, obj: dict) -> None:
    path.write_text(json.dumps(obj, indent=1) + "\n")
    print(f"wrote {path.relative_to(ROOT)} ({path.stat().st_size} bytes)")


def main() -> None:
    O.build_oracle(with_ref=True)
    ref = O.ref()

    # --- the reference's whole driver, 25y -------------------------------------
    mk, sw = market_inputs(n_periods=50)
    n_paths, dt, expiry = 64, 0.01, 25.0
    n_steps = 2500
    ee_ref = np.zeros(51)
    ref.ref_calculate_exposure_cpu(ee_ref, sw.notional, sw.strike, expiry, 0.5, sw.accrual, mk.spot, mk.drift,
                                   mk.vol.ravel(), n_paths, dt)
    normals = O.curand_normals_double(n_paths * n_steps * 3, seed=1234).reshape(n_paths, n_steps, 3)
    ee_orc = O.expected_exposure(O.exposure_paths(mk, sw, n_steps, dt, normals))
    err = np.max(np.abs(ee_orc - ee_ref) / np.maximum(np.abs(ee_ref), 1e-300))
    print(f"25y driver: max rel diff oracle vs reference = {err:.3e}")
    assert err < 1e-13, err
    dump(HERE / "ref_driver_25y.json", {
        "source": "reference calculateExposureCPU<double> (simulation_cpu.h:350), unmodified",
        "normals": {"generator": "curand host CURAND_RNG_PSEUDO_DEFAULT (XORWOW)", "seed": 1234,
                    "call": "curandGenerateNormalDouble(count, 0.0, 1.0)", "count": n_paths * n_steps * 3,
                    "layout": "[path][step][factor]"},
        "n_paths": n_paths, "n_steps": n_steps, "dt": dt, "expiry": expiry, "dtau": 0.5,
        "notional": sw.notional, "strike": sw.strike,
        "spot": mk.spot.tolist(), "vol": mk.vol.ravel().tolist(), "drift": mk.drift.tolist(),
        "accrual": sw.accrual.tolist(),
        "ee": ee_ref.tolist(),
    })

    # --- the reference driver's own workload -----------------------------------
    src = (REFERENCE / "simulation_gpu_testing.cpp").read_text()
    spot, vol = driver_array(src, "spot_rates"), driver_array(src, "volatilities")
    drift, accrual = driver_array(src, "drifts"), driver_array(src, "accrual")
    # the driver's double copies hold the same values
    for a, b in ((spot, "spot_rates_d"), (vol, "volatilities_d"), (drift, "drifts_d"), (accrual, "accrual_d")):
        assert np.array_equal(a, driver_array(src, b)), b
    assert spot.shape == (51,) and vol.shape == (153,) and drift.shape == (51,) and accrual.shape == (51,)
    m = re.search(r"InterestRateSwap<real>\s+payOff\([^,]+,[^,]+,[^,]+,\s*([0-9.eE+-]+)\s*,\s*([0-9.eE+-]+)", src)
    notional, strike = float(m.group(1)), float(m.group(2))
    expiry = float(re.search(r"const real expiry\s*=\s*([0-9.]+)", src).group(1))
    dtau = float(re.search(r"const real dtau\s*=\s*([0-9.]+)", src).group(1))
    dt = 0.01  # the driver's default -dt
    n_paths, n_steps = 5000, int(round(expiry / dt))
    ee_ref = np.zeros(51)
    ref.ref_calculate_exposure_cpu(ee_ref, notional, strike, expiry, dtau, accrual, spot, drift, vol, n_paths, dt)
    mk = Market(n_tenor=51, dtau=dtau, spot=spot, vol=vol.reshape(3, 51), drift=drift)
    sw = Swap(notional=notional, strike=strike, n_tenor=51, dtau=dtau, accrual=accrual)
    normals = O.curand_normals_double(n_paths * n_steps * 3, seed=1234).reshape(n_paths, n_steps, 3)
    x_orc = O.exposure_paths(mk, sw, n_steps, dt, normals)
    ee_orc = O.expected_exposure(x_orc)
    err = np.max(np.abs(ee_orc - ee_ref) / np.maximum(np.abs(ee_ref), 1e-300))
    print(f"driver's own workload: EE[0] = {ee_ref[0]:.6f}, max rel diff oracle vs reference = {err:.3e}")
    assert err < 1e-13, err
    keep = 16
    x_ref = np.zeros((keep, 51))
    ee_keep = np.zeros(51)
    rc = ref.ref_exposure_paths(n_steps, spot, vol, drift, accrual, notional, strike, keep,
                               np.ascontiguousarray(normals[:keep]).ravel(), x_ref.ravel(), ee_keep)
    assert rc == 0
    assert np.array_equal(x_orc[:keep], x_ref), np.max(np.abs(x_orc[:keep] - x_ref))
    dump(HERE / "ref_driver_own_market.json", {
        "source": "reference calculateExposureCPU<double> (simulation_cpu.h:350), unmodified, on the driver's own "
                  "inputs (simulation_gpu_testing.cpp:36-123, swap :215); exposures_first_paths from "
                  "__generatePaths_kernel_cpu / __calculateExposure_kernel (simulation_cpu.h:188,270)",
        "normals": {"generator": "curand host CURAND_RNG_PSEUDO_DEFAULT (XORWOW)", "seed": 1234,
                    "call": "curandGenerateNormalDouble(count, 0.0, 1.0)", "count": n_paths * n_steps * 3,
                    "layout": "[path][step][factor]"},
        "n_paths": n_paths, "n_steps": n_steps, "dt": dt, "expiry": expiry, "dtau": dtau,
        "notional": notional, "strike": strike,
        "spot": spot.tolist(), "vol": vol.tolist(), "drift": drift.tolist(), "accrual": accrual.tolist(),
        "ee": ee_ref.tolist(),
        "exposures_first_paths": x_ref.tolist(),
    })

    # --- the reference's per-path functions, 10y, zeroed numeraires -------------
    mk, sw = market_inputs(n_periods=20)
    n_paths, n_steps = 128, 1000
    normals = O.curand_normals_double(n_paths * n_steps * 3, seed=1234).reshape(n_paths, n_steps, 3)
    x_ref = np.zeros((n_paths, 51))
    ee_ref = np.zeros(51)
    rc = ref.ref_exposure_paths(n_steps, mk.spot, mk.vol.ravel(), mk.drift, sw.accrual, sw.notional, sw.strike,
                                n_paths, normals.ravel(), x_ref.ravel(), ee_ref)
    assert rc == 0
    x_orc = O.exposure_paths(mk, sw, n_steps, dt, normals)
    ee_orc = O.expected_exposure(x_orc)
    assert np.array_equal(x_orc, x_ref), np.max(np.abs(x_orc - x_ref))
    assert np.max(np.abs(ee_orc - ee_ref)) <= 1e-13 * np.max(np.abs(ee_ref))
    print("10y blocks: oracle exposures equal the reference's bit for bit")
    keep = 16
    dump(HERE / "ref_blocks_10y.json", {
        "source": "reference __generatePaths_kernel_cpu / __calculateExposure_kernel / "
                  "__calculateExpectedExposure_kernel (simulation_cpu.h:188,270,336), numeraires zeroed",
        "normals": {"generator": "curand host CURAND_RNG_PSEUDO_DEFAULT (XORWOW)", "seed": 1234,
                    "call": "curandGenerateNormalDouble(count, 0.0, 1.0)", "count": n_paths * n_steps * 3,
                    "layout": "[path][step][factor]"},
        "n_paths": n_paths, "n_steps": n_steps, "dt": dt, "dtau": 0.5,
        "notional": sw.notional, "strike": sw.strike,
        "spot": mk.spot.tolist(), "vol": mk.vol.ravel().tolist(), "drift": mk.drift.tolist(),
        "accrual": sw.accrual.tolist(),
        "ee": ee_ref.tolist(),
        "exposures_first_paths": x_ref[:keep].tolist(),
    })


if __name__ == "__main__":
    main()
