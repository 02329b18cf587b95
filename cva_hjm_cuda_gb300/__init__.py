"""GB300-native Monte Carlo HJM exposure / CVA engine.

A from-scratch implementation, for one NVIDIA GB300 (sm_103a), of the Monte
Carlo path of mahsanchez/cva_hjm_cuda: multi-factor HJM forward-curve
evolution in the Musiela parameterisation, interest-rate-swap exposure on the
0.5y grid, EE / PFE reduction and the CVA sum, plus a mixed-precision form and
a pathwise adjoint.  The kernels and the C ABI live in ``csrc/`` and build to
``lib/libhjmcva.so``; this package holds the Python host mirror used by tests
and benchmarks.
"""
from .market import Market, RunConfig, Swap, quantile_rank  # noqa: F401

__all__ = ["Market", "Swap", "RunConfig", "quantile_rank", "HJMEngine", "calculate_exposure_gpu"]


def __getattr__(name):
    # the engine loads libhjmcva.so lazily so that importing the package works on a CPU-only host
    if name in ("HJMEngine", "calculate_exposure_gpu", "Valuation", "Sensitivities"):
        from . import engine

        return getattr(engine, name)
    raise AttributeError(name)
