"""Shared fixtures.  GPU tests carry @pytest.mark.gpu and need a CUDA device;
everything else runs on the CPU (the oracle, host logic, library exports)."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
TESTS = Path(__file__).resolve().parent
for p in (str(ROOT), str(TESTS)):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = TESTS / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libhjmcva.so")
    config.addinivalue_line("markers", "slow: long-running (full-size workloads)")


def load_golden(name: str) -> dict:
    return json.loads((GOLDEN / name).read_text())


@pytest.fixture(scope="session")
def golden_10y():
    return load_golden("ref_blocks_10y.json")


@pytest.fixture(scope="session")
def golden_25y():
    return load_golden("ref_driver_25y.json")


@pytest.fixture(scope="session")
def golden_own():
    """The reference driver's own workload (its curve, PCA volatility table,
    drift table, irregular accruals; N = 10, K = 6.7%, 25y; 5,000 paths)."""
    return load_golden("ref_driver_own_market.json")


def market_from_golden(g: dict):
    from cva_hjm_cuda_gb300.market import Market, Swap

    mk = Market(n_tenor=51, dtau=g["dtau"], spot=np.array(g["spot"]), vol=np.array(g["vol"]).reshape(3, 51),
                drift=np.array(g["drift"]))
    sw = Swap(notional=g["notional"], strike=g["strike"], n_tenor=51, dtau=g["dtau"], accrual=np.array(g["accrual"]))
    return mk, sw


def _have_gpu() -> bool:
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.fixture(scope="session")
def engine():
    if not _have_gpu():
        pytest.skip("no CUDA device")
    from cva_hjm_cuda_gb300.engine import HJMEngine

    e = HJMEngine(0)
    yield e
    e.close()
