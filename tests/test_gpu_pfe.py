"""The PFE selection (launch_pfe: 11-bit radix passes over the exposure
store, then the few candidates left copied out and ranked in shared memory)
against numpy's k-th smallest of the stored exposures, bit for bit.

* a continuous column: the candidates are compacted after two digits;
* a payer swap far out of the money (strike 20%): most exposures are zero,
  the candidates stay many and the global passes finish the selection;
* 100 and 2,000 paths: compacted after the first digit, ties included (the
  first date's exposures are all equal);
* quantiles at both ends (k = 1 and k = n; the quantile must be below 1)
  and in between;
* FP64 keys and the mixed valuation's FP32 keys.
"""
from __future__ import annotations

import numpy as np
import pytest

from cva_hjm_cuda_gb300.market import Market, RunConfig, Swap

pytestmark = pytest.mark.gpu


def _kth(col: np.ndarray, q: float) -> float:
    n = col.size
    k = min(max(int(np.ceil(q * n - 1e-7)), 1), n)  # as the library's k
    return float(np.partition(col, k - 1)[k - 1])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("n_paths,strike,q", [(65_536, 0.025, 0.975), (65_536, 0.2, 0.975), (100, 0.025, 0.975),
                                              (2_000, 0.025, 0.5), (4_099, 0.025, 1e-9), (4_099, 0.025, 1.0 - 1e-9),
                                              (30_000, 0.03, 0.9)],
                         ids=["continuous", "mostly-zero", "100-paths", "2000-paths-median", "k=1", "k=n",
                              "q=0.9"])
def test_pfe_is_the_kth_smallest_exposure(engine, precision, n_paths, strike, q):
    engine.set_market(Market())
    engine.set_swap(Swap(strike=strike))
    engine.keep_exposures(True)
    try:
        v = engine.run(RunConfig(n_paths=n_paths, pfe_quantile=q, seed=11), precision)
        x = engine.exposures()
    finally:
        engine.keep_exposures(False)
    for j in range(x.shape[0]):
        col = x[j].astype(np.float32) if precision == "mixed" else x[j]
        assert v.pfe[j] == _kth(col, q), (j, v.pfe[j], _kth(col, q))
    if strike == 0.2:
        assert np.mean(x[1:] == 0.0) > 0.975  # the ties the global passes resolve
