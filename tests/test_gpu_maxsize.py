"""Maximum sizes: one call of 2^28 paths, against the oracle and against its halves.

The reference's GPU path keeps its normals in one buffer with an ``int``
count (simulation_gpu.cu:195-216), which overflows past ~715,000 paths x 1,000
steps x 3 factors; here the normals are made in registers, a call takes up to
2^31 paths and the exposure store is addressed with 64-bit offsets.  At
268,435,456 paths x 1,000 steps (10y swap, 21 dates) the FP64 store holds
5.6e9 values (45 GB; byte offsets pass 2^32 from date 2 on and element
offsets pass 2^31 from date 8 on) in a launch of 4,194,304 CTAs.

* FP64 with PFE(97.5%): paths at the start, around the 2^27 split, and in
  the last CTA are read back alone (hjm_get_exposure_paths) and re-priced by
  the oracle on their own normals (1e-10 relative, 1e-13 of the exposure
  scale); the EE and CVA equal the mean of the two half-runs' (path offsets
  0 and 2^27; 1e-12 relative), and each date's PFE lies between the halves'
  (the q-quantile of a union of two equal sets lies between theirs).
* mixed precision on the same paths: EE and CVA within 1e-4 of the FP64 run's,
  and the sampled paths within 1e-4 of the exposure scale from the oracle.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle_lib as O
from cva_hjm_cuda_gb300.market import Market, RunConfig, Swap

pytestmark = pytest.mark.gpu

N = 1 << 28
HALF = N >> 1
RUN = 64
STARTS = [0, 4096 + 17, HALF - RUN // 2, HALF + 1000, N - 3 * 64 - 5, N - RUN]


@pytest.fixture(scope="module")
def big_engine():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from cva_hjm_cuda_gb300.engine import HJMEngine

    e = HJMEngine(0)
    e.set_market(Market())
    e.set_swap(Swap())
    yield e
    e.close()  # frees the 45 GB store before the later test files


def _oracle_slices(engine, cfg, n_dates):
    mk, sw = Market(), Swap()
    out = []
    for s0 in STARTS:
        normals = engine.dump_normals(RUN, cfg.n_steps, cfg.seed, path_offset=s0)
        out.append(O.exposure_paths(mk, sw, cfg.n_steps, cfg.dt, normals)[:, :n_dates])
    return np.concatenate(out)


def _device_slices(engine):
    return np.concatenate([engine.exposure_paths(s0, RUN).T for s0 in STARTS])


@pytest.fixture(scope="module")
def fp64_run(big_engine):
    cfg = RunConfig(n_paths=N, n_steps=1000, dt=0.01, seed=1234)
    v = big_engine.run(cfg, "fp64")
    assert big_engine.remainder_form() == "response"
    got = _device_slices(big_engine)
    return cfg, v, got


def test_fp64_2pow28_paths_sampled_vs_oracle(big_engine, fp64_run):
    cfg, v, got = fp64_run
    want = _oracle_slices(big_engine, cfg, 21)
    scale = np.max(np.abs(want))
    err = np.abs(got - want)
    bad = (err > 1e-10 * np.abs(want)) & (err > 1e-13 * scale)
    assert not np.any(bad), f"max rel err {np.max(err / np.maximum(np.abs(want), 1e-300)):.3e}"


def test_fp64_2pow28_paths_equals_its_halves(big_engine, fp64_run):
    cfg, v, _ = fp64_run
    halves = []
    for off in (0, HALF):
        c = RunConfig(n_paths=HALF, n_steps=1000, dt=0.01, seed=1234, path_offset=off)
        halves.append(big_engine.run(c, "fp64"))
    a, b = halves
    ee = 0.5 * (a.ee[:21] + b.ee[:21])
    np.testing.assert_allclose(v.ee[:21], ee, rtol=1e-12, atol=1e-12 * np.max(ee))
    np.testing.assert_allclose(v.cva, 0.5 * (a.cva + b.cva), rtol=1e-12)
    lo = np.minimum(a.pfe[:21], b.pfe[:21])
    hi = np.maximum(a.pfe[:21], b.pfe[:21])
    assert np.all(v.pfe[:21] >= lo) and np.all(v.pfe[:21] <= hi)
    assert np.all(v.pfe[1:20] > 0)


def test_mixed_2pow28_paths_vs_fp64_and_oracle(big_engine, fp64_run):
    cfg, v64, _ = fp64_run
    vmx = big_engine.run(cfg, "mixed")
    ee64 = v64.ee[:21]
    # (the last date's exposure is zero on every path)
    np.testing.assert_allclose(vmx.ee[:21], ee64, rtol=1e-4, atol=1e-12 * np.max(ee64))
    assert abs(vmx.cva - v64.cva) < 1e-4 * v64.cva
    got = _device_slices(big_engine)
    want = _oracle_slices(big_engine, cfg, 21)
    assert np.max(np.abs(got - want)) <= 1e-4 * np.max(np.abs(want))


def test_path_count_limit_and_slice_bounds(big_engine):
    from cva_hjm_cuda_gb300._lib import HJMError

    # more than 2^31 paths in one call: rejected before any device work
    with pytest.raises(HJMError) as e:
        big_engine.run(RunConfig(n_paths=(1 << 31) + 1, n_steps=1000, dt=0.01, seed=1234), "fp64")
    assert e.value.status == 1 and "2^31" in str(e.value)  # HJM_ERR_INVALID_ARGUMENT
    # a slice must lie inside the last run's paths
    big_engine.run(RunConfig(n_paths=1000, n_steps=1000, dt=0.01, seed=1234), "fp64")
    for begin, n in ((-1, 10), (995, 10), (0, 0), (0, 1001)):
        with pytest.raises(HJMError):
            big_engine.exposure_paths(begin, n)
    x = big_engine.exposure_paths(990, 10)
    assert x.shape == (21, 10) and np.all(x >= 0)
