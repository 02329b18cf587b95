"""Device normals at scale, and the host-side out-of-memory path.

* The normals the path kernels draw (Philox4x32-10, Box-Muller on 24-bit
  uniforms in FP32 with the SFU): 16.8 million of them, dumped through
  hjm_dump_normals, against N(0, 1): the first four moments, a
  Kolmogorov-Smirnov test, the tail mass beyond 3 and 4 sigma, and the
  truncation at sqrt(-2 ln 2^-24) = 5.768 sigma that the 24-bit uniforms
  imply (N(0, 1) puts 8e-9 of its mass beyond it: 0.13 draws expected here).
* A context whose memory cap (hjm_ctx_set_memory_limit) is below what a
  valuation needs reports HJM_ERR_OUT_OF_MEMORY with a message, allocates
  nothing, and runs normally once the cap is lifted.  The failure is made on
  the host; no GPU fault is involved.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from cva_hjm_cuda_gb300 import _lib
from cva_hjm_cuda_gb300.market import Market, RunConfig, Swap

pytestmark = pytest.mark.gpu


def test_device_normals_distribution(engine):
    n_paths, n_steps = 5600, 1000  # 16.8e6 draws
    z = engine.dump_normals(n_paths, n_steps, seed=1234).ravel()
    n = z.size
    mean, var = float(z.mean()), float(z.var())
    zc = z - mean
    skew = float(np.mean(zc**3)) / var**1.5
    kurt = float(np.mean(zc**4)) / var**2
    # five standard errors of each estimator under N(0, 1)
    assert abs(mean) < 5.0 / math.sqrt(n), mean
    assert abs(var - 1.0) < 5.0 * math.sqrt(2.0 / n), var
    assert abs(skew) < 5.0 * math.sqrt(6.0 / n), skew
    assert abs(kurt - 3.0) < 5.0 * math.sqrt(24.0 / n), kurt
    # Kolmogorov-Smirnov on a 2M subsample (the exact CDF via erf)
    from scipy import stats

    sub = z[:: n // 2_000_000][:2_000_000]
    ks = stats.kstest(sub, "norm")
    assert ks.pvalue > 1e-4, ks
    # tail mass: counts beyond 3 and 4 sigma within five Poisson standard deviations
    for a in (3.0, 4.0):
        p = math.erfc(a / math.sqrt(2.0))
        expect = p * n
        got = int(np.count_nonzero(np.abs(z) > a))
        assert abs(got - expect) < 5.0 * math.sqrt(expect) + 1, (a, got, expect)
    # the 24-bit uniforms bound the radius: |z| <= sqrt(-2 ln 2^-24)
    cut = math.sqrt(-2.0 * math.log(2.0**-24))
    assert float(np.max(np.abs(z))) <= cut * (1.0 + 1e-6)
    assert np.all(np.isfinite(z))


def test_memory_cap_reports_out_of_memory_and_context_recovers(engine):
    mk, sw = Market(), Swap()
    engine.set_market(mk)
    engine.set_swap(sw)
    small = RunConfig(n_paths=4096, seed=77)
    ref_small = engine.run(small, "fp64")
    held = engine.memory_in_use()
    assert held > 0
    big = RunConfig(n_paths=1 << 20, seed=77)
    engine.set_memory_limit(held)  # no growth allowed
    try:
        with pytest.raises(_lib.HJMError) as ei:
            engine.run(big, "fp64")  # the PFE store of 1M paths does not fit
        assert ei.value.status == 4  # HJM_ERR_OUT_OF_MEMORY
        assert "cudaErrorMemoryAllocation" in str(ei.value) or "out of memory" in str(ei.value)
        assert engine.memory_in_use() == held  # nothing freed, nothing allocated
        # a run that fits the buffers already held still runs under the cap
        again = engine.run(small, "fp64")
        np.testing.assert_array_equal(again.ee, ref_small.ee)
        assert again.cva == ref_small.cva
    finally:
        engine.set_memory_limit(0)
    v = engine.run(big, "fp64")
    assert np.all(np.isfinite(v.ee)) and v.cva > 0
    assert engine.memory_in_use() > held
    with pytest.raises(_lib.HJMError) as ei:
        engine.set_memory_limit(-1)
    assert ei.value.status == 1
