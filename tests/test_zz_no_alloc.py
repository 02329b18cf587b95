"""hjm_run_static: the allocation-free entry point.

Some callers cannot allocate device memory once they are running: a risk
server whose pool allocator already owns the GPU, a pricing plugin loaded into
such a process, or a latency-bound loop that cannot take the device-wide
synchronisation a cudaMalloc/cudaFree may cause.  hjm_run_static serves them
from a fixed static device scratch (at most HJM_STATIC_MAX_PATHS paths, EE and
CVA only).  This test calls it through the C ABI twice in a row and checks it
against the context-based hjm_run, within the FP64 parity tolerance of the
other GPU tests, and checks that oversize runs are refused with a clear error.

The file name makes pytest collect it last; it must also pass on its own in a
fresh process (the first call on the device does the scratch set-up).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from cva_hjm_cuda_gb300 import _lib
from cva_hjm_cuda_gb300.market import Market, RunConfig, Swap

pytestmark = pytest.mark.gpu

FP64_RTOL = 1e-10
MIXED_RTOL = 1e-4


def _have_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _run_static(lib, mk, sw, cfg, precision):
    ee, cva = np.zeros(mk.n_tenor), np.zeros(3)
    st = lib.hjm_run_static(None, mk.n_tenor, mk.dtau, _dp(mk.spot), _dp(np.ascontiguousarray(mk.vol.ravel())),
                            _dp(mk.drift), sw.notional, sw.strike, _dp(sw.accrual), 1 if sw.payer else 0,
                            cfg.n_paths, cfg.n_steps, cfg.dt, cfg.seed, cfg.path_offset, _lib.PRECISION[precision],
                            cfg.hazard, cfg.recovery, _dp(ee), _dp(cva))
    return st, ee, cva


@pytest.mark.skipif(not _have_gpu(), reason="no CUDA device")
@pytest.mark.parametrize("precision,rtol", [("fp64", FP64_RTOL), ("mixed", MIXED_RTOL)])
def test_static_entry_matches_hjm_run_twice(precision, rtol):
    from cva_hjm_cuda_gb300.engine import HJMEngine

    lib = _lib.load()
    mk, sw = Market(), Swap()
    cfg = RunConfig(n_paths=50_000, n_steps=1000, dt=0.01, seed=4321, path_offset=7)
    with HJMEngine(0) as eng:
        eng.set_market(mk)
        eng.set_swap(sw)
        ref = eng.run(cfg, precision, pfe=False)
    for call in range(2):
        st, ee, cva = _run_static(lib, mk, sw, cfg, precision)
        assert st == 0, lib.hjm_last_error(None)
        np.testing.assert_allclose(ee, ref.ee, rtol=rtol, atol=0, err_msg=f"EE, call {call}")
        assert abs(cva[0] - ref.cva) <= rtol * abs(ref.cva), f"CVA, call {call}"
        assert abs(cva[1] - ref.cva_stderr) <= 1e-6 * ref.cva_stderr
        assert abs(cva[2] - ref.dcva_dhazard) <= rtol * abs(ref.dcva_dhazard)


@pytest.mark.skipif(not _have_gpu(), reason="no CUDA device")
@pytest.mark.parametrize("case", ["bumpy-table", "table-beyond-static", "reference-pca-table"])
def test_static_fp64_response_and_fallback_match_hjm_run(case):
    """FP64 static runs take a response form when its table fits the static
    array: the polynomial one for quadratic factors (the test above) and for
    cubic factors with a residual table (the reference's PCA table), the
    volatility-table one for any other table (bumpy-table), the convected step
    when neither fits (1,000 steps per date); all equal hjm_run within 1e-10."""
    from cva_hjm_cuda_gb300.engine import HJMEngine

    lib = _lib.load()
    if case == "bumpy-table":
        mk = Market(vol=Market().vol * (1.0 + 0.1 * np.cos(np.arange(51) / 7.0))[None, :])
        cfg = RunConfig(n_paths=20_000, seed=8)
    elif case == "reference-pca-table":
        # cubic factors with a residual table: the cubic response form in the static array
        import json
        from pathlib import Path

        g = json.loads((Path(__file__).parent / "golden" / "ref_driver_own_market.json").read_text())
        mk = Market(vol=np.array(g["vol"]).reshape(3, 51))
        cfg = RunConfig(n_paths=20_000, seed=8)
    else:
        mk = Market()
        cfg = RunConfig(n_paths=20_000, n_steps=20000, dt=0.0005, seed=8)
    sw = Swap()
    with HJMEngine(0) as eng:
        eng.set_market(mk)
        eng.set_swap(sw)
        ref = eng.run(cfg, "fp64", pfe=False)
    st, ee, cva = _run_static(lib, mk, sw, cfg, "fp64")
    assert st == 0, lib.hjm_last_error(None)
    np.testing.assert_allclose(ee, ref.ee, rtol=FP64_RTOL, atol=0)
    assert abs(cva[0] - ref.cva) <= FP64_RTOL * abs(ref.cva)


@pytest.mark.skipif(not _have_gpu(), reason="no CUDA device")
@pytest.mark.parametrize("precision,rtol", [("fp64", FP64_RTOL), ("mixed", MIXED_RTOL)])
def test_static_entry_matches_oracle(precision, rtol):
    """hjm_run_static against the oracle directly (5,000 paths of the 10y swap), on the
    device's own normals: its parity does not rest on hjm_run."""
    import oracle_lib as O
    from cva_hjm_cuda_gb300.engine import HJMEngine

    lib = _lib.load()
    mk, sw = Market(), Swap()
    cfg = RunConfig(n_paths=5000, n_steps=1000, dt=0.01, seed=1234, path_offset=3)
    with HJMEngine(0) as eng:
        normals = eng.dump_normals(cfg.n_paths, cfg.n_steps, cfg.seed, cfg.path_offset)
    x = O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)
    ee = O.expected_exposure(x)
    cva, dcva = O.cva(ee, 21, mk.dtau, cfg.hazard, cfg.recovery)
    st, ee_s, cva_s = _run_static(lib, mk, sw, cfg, precision)
    assert st == 0, lib.hjm_last_error(None)
    np.testing.assert_allclose(ee_s[:20], ee[:20], rtol=rtol, atol=0)
    assert np.all(ee_s[20:] == 0.0)
    assert abs(cva_s[0] - cva) <= rtol * cva
    assert abs(cva_s[2] - dcva) <= rtol * abs(dcva)


@pytest.mark.skipif(not _have_gpu(), reason="no CUDA device")
@pytest.mark.parametrize("market", ["quadratic", "reference-pca-table"])
def test_static_mixed_runs_the_decomposition_like_hjm_run(market):
    """With quadratic factors, or the reference driver's PCA table (cubic up to
    a residual), the static mixed run takes the same polynomial form as
    hjm_run and gives hjm_run's results to rounding."""
    from conftest import load_golden
    from cva_hjm_cuda_gb300.engine import HJMEngine

    lib = _lib.load()
    if market == "quadratic":
        mk = Market()
    else:
        mk = Market(vol=np.array(load_golden("ref_driver_own_market.json")["vol"]).reshape(3, 51))
    sw = Swap()
    cfg = RunConfig(n_paths=30_000, seed=99)
    with HJMEngine(0) as eng:
        eng.set_market(mk)
        eng.set_swap(sw)
        assert eng.vol_decomposition() > 0
        ref = eng.run(cfg, "mixed", pfe=False)
    st, ee, cva = _run_static(lib, mk, sw, cfg, "mixed")
    assert st == 0, lib.hjm_last_error(None)
    np.testing.assert_allclose(ee, ref.ee, rtol=1e-12, atol=0)
    assert abs(cva[0] - ref.cva) <= 1e-12 * ref.cva


@pytest.mark.skipif(not _have_gpu(), reason="no CUDA device")
def test_static_entry_rejects_oversize_runs():
    lib = _lib.load()
    mk, sw = Market(), Swap()
    cfg = RunConfig(n_paths=_lib.STATIC_MAX_PATHS + 1)
    st, _, _ = _run_static(lib, mk, sw, cfg, "fp64")
    assert st == 1  # HJM_ERR_INVALID_ARGUMENT
    assert b"HJM_STATIC_MAX_PATHS" in lib.hjm_last_error(None)
