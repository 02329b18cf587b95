"""The C ABI library: it loads, exports every symbol include/*.h declares, and
rejects bad calls without a GPU."""
from __future__ import annotations

import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

from cva_hjm_cuda_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]


def _declared_c_functions() -> set[str]:
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        src = h.read_text()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(hjm_\w+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def lib():
    if not _lib.LIB_PATH.exists():
        from cva_hjm_cuda_gb300 import build

        build.build()
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    declared = _declared_c_functions()
    assert declared, "no declarations found"
    out = subprocess.run(["nm", "-D", "--defined-only", str(_lib.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (\w+)", out))
    missing = declared - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    assert set(_lib.EXPORTED) == declared
    # the C++ drop-in overloads of simulation_gpu.h:12,14, with the reference's mangled names
    assert "_Z25calculateExposureMultiGPUPd16InterestRateSwapIdES_S_S_S_diid" in exported
    assert "_Z25calculateExposureMultiGPUPf16InterestRateSwapIfES_S_S_S_fiif" in exported


def test_version_and_null_context(lib):
    assert lib.hjm_version().startswith(b"hjmcva")
    st = lib.hjm_set_market(None, 51, 0.5, None, None, 3, None)
    assert st == 1
    assert b"null context" in lib.hjm_last_error(None)
    assert lib.hjm_ctx_destroy(None) == 0


def test_context_creation_reports_missing_device(lib):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    h = C.c_void_p()
    st = lib.hjm_ctx_create(0, C.byref(h))
    assert st == 6  # HJM_ERR_NO_DEVICE
    assert h.value is None
    assert lib.hjm_last_error(None)


def test_product_has_no_cpu_fallback():
    """The package's engine module never imports the oracle."""
    for f in (ROOT / "cva_hjm_cuda_gb300").rglob("*.py"):
        text = f.read_text()
        assert "oracle" not in text.replace("oracle is", ""), f"{f} references the oracle"
