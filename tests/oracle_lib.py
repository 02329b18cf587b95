"""ctypes bindings for the oracle (test infrastructure).

Loads ``oracle/_build/libhjm_oracle.so`` (the C restatement, built anywhere by
``make -C oracle oracle``), optionally ``oracle/_ref/libhjm_ref.so`` (the
reference's own simulation_cpu.h compiled where the reference tree exists),
and the cuRAND host generator, used only to reproduce the reference's own
normal draws (cuRAND host XORWOW, seed 1234) and as a Philox known-answer
source.  Nothing in the product imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
ORACLE_DIR = ROOT / "oracle"
ORACLE_SO = ORACLE_DIR / "_build" / "libhjm_oracle.so"
REF_SO = ORACLE_DIR / "_ref" / "libhjm_ref.so"

_dp = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build_oracle(with_ref: bool = False) -> None:
    """Build the oracle and, with with_ref, the reference's own CPU path where
    its source tree is present (the Makefile's REF, from HJM_REFERENCE_DIR)."""
    targets = ["oracle"] + (["ref-if-present"] if with_ref else [])
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR), *targets], check=True)


_oracle = None


def oracle() -> C.CDLL:
    global _oracle
    if _oracle is None:
        if not ORACLE_SO.exists():
            build_oracle()
        lib = C.CDLL(str(ORACLE_SO))
        lib.oracle_exposure_paths.restype = C.c_int
        lib.oracle_exposure_paths.argtypes = [
            C.c_int, C.c_double, C.c_double, C.c_int, _dp, _dp, _dp, _dp,
            C.c_double, C.c_double, C.c_double, C.c_int, _dp, _dp,
        ]
        lib.oracle_exposure_paths_scheme.restype = C.c_int
        lib.oracle_exposure_paths_scheme.argtypes = [
            C.c_int, C.c_int, C.c_double, C.c_double, C.c_int, _dp, _dp, _dp, _dp,
            C.c_double, C.c_double, C.c_double, C.c_int, _dp, _dp,
        ]
        lib.oracle_exposure_paths_netting.restype = C.c_int
        lib.oracle_exposure_paths_netting.argtypes = [
            C.c_int, C.c_double, C.c_double, C.c_int, _dp, _dp, _dp, _dp, _dp, C.c_int, _dp, _dp,
        ]
        lib.oracle_expected_exposure.restype = None
        lib.oracle_expected_exposure.argtypes = [_dp, C.c_int, C.c_int, _dp]
        lib.oracle_trapezoid_drift.restype = None
        lib.oracle_trapezoid_drift.argtypes = [_dp, C.c_int, C.c_int, C.c_double, _dp]
        lib.oracle_cva.restype = C.c_double
        lib.oracle_cva.argtypes = [_dp, C.c_int, C.c_double, C.c_double, C.c_double, C.POINTER(C.c_double)]
        lib.oracle_cva_paths.restype = None
        lib.oracle_cva_paths.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, _dp]
        lib.oracle_pfe.restype = None
        lib.oracle_pfe.argtypes = [_dp, C.c_int, C.c_int, C.c_int, C.c_double, _dp]
        lib.oracle_quantile_rank.restype = C.c_long
        lib.oracle_quantile_rank.argtypes = [C.c_double, C.c_long]
        lib.oracle_philox4x32_10.restype = None
        lib.oracle_philox4x32_10.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        lib.oracle_normals_host.restype = None
        lib.oracle_normals_host.argtypes = [C.c_uint64, C.c_uint64, C.c_int, C.c_int, _dp]
        lib.oracle_run_mt.restype = C.c_int
        lib.oracle_run_mt.argtypes = [
            C.c_int, C.c_double, C.c_double, C.c_int, _dp, _dp, _dp, _dp,
            C.c_double, C.c_double, C.c_double, C.c_long, C.c_uint64, C.c_uint64, C.c_int, _dp,
        ]
        _oracle = lib
    return _oracle


_ref = None


def ref_available() -> bool:
    """Whether the reference's CPU path is built (or can be: its tree is present)."""
    if not REF_SO.exists():
        try:
            build_oracle(with_ref=True)
        except (OSError, subprocess.CalledProcessError):
            return False
    return REF_SO.exists()


def ref() -> C.CDLL:
    """The reference's own CPU path (only where the reference tree is present)."""
    global _ref
    if _ref is None:
        if not ref_available():
            raise OSError("the reference's CPU path is not built and its source tree is absent")
        lib = C.CDLL(str(REF_SO))
        lib.ref_exposure_paths.restype = C.c_int
        lib.ref_exposure_paths.argtypes = [C.c_int, _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_int, _dp, _dp, _dp]
        lib.ref_calculate_exposure_cpu.restype = C.c_int
        lib.ref_calculate_exposure_cpu.argtypes = [
            _dp, C.c_double, C.c_double, C.c_double, C.c_double, _dp, _dp, _dp, _dp, C.c_int, C.c_double,
        ]
        _ref = lib
    return _ref


# ---------------------------------------------------------------------------
# oracle wrappers
# ---------------------------------------------------------------------------

def exposure_paths(market, swap, n_steps: int, dt: float, normals: np.ndarray) -> np.ndarray:
    """Per-path exposures [n_paths][n_tenor] from normals [n_paths][n_steps][3]."""
    normals = np.ascontiguousarray(normals, dtype=np.float64)
    n_paths = normals.shape[0]
    assert normals.shape == (n_paths, n_steps, 3)
    out = np.zeros((n_paths, market.n_tenor), dtype=np.float64)
    rc = oracle().oracle_exposure_paths(
        market.n_tenor, market.dtau, dt, n_steps, market.spot, market.vol.ravel(), market.drift,
        swap.accrual, swap.notional, swap.strike, swap.sign, n_paths, normals.ravel(), out.ravel(),
    )
    if rc != 0:
        raise ValueError(f"oracle_exposure_paths rejected its arguments (rc={rc})")
    return out


def exposure_paths_pc(market, swap, n_steps: int, dt: float, normals: np.ndarray) -> np.ndarray:
    """Per-path exposures under the predictor-corrector scheme."""
    normals = np.ascontiguousarray(normals, dtype=np.float64)
    n_paths = normals.shape[0]
    out = np.zeros((n_paths, market.n_tenor), dtype=np.float64)
    rc = oracle().oracle_exposure_paths_scheme(
        1, market.n_tenor, market.dtau, dt, n_steps, market.spot, market.vol.ravel(), market.drift,
        swap.accrual, swap.notional, swap.strike, swap.sign, n_paths, normals.ravel(), out.ravel(),
    )
    if rc != 0:
        raise ValueError(f"oracle_exposure_paths_scheme rejected its arguments (rc={rc})")
    return out


def exposure_paths_netting(market, payA, payB, n_steps: int, dt: float, normals: np.ndarray) -> np.ndarray:
    """Per-path netted exposures for per-date payoff vectors (cash flow D (payA L - payB))."""
    normals = np.ascontiguousarray(normals, dtype=np.float64)
    n_paths = normals.shape[0]
    out = np.zeros((n_paths, market.n_tenor), dtype=np.float64)
    rc = oracle().oracle_exposure_paths_netting(
        market.n_tenor, market.dtau, dt, n_steps, market.spot, market.vol.ravel(), market.drift,
        np.ascontiguousarray(payA, dtype=np.float64), np.ascontiguousarray(payB, dtype=np.float64),
        n_paths, normals.ravel(), out.ravel(),
    )
    if rc != 0:
        raise ValueError(f"oracle_exposure_paths_netting rejected its arguments (rc={rc})")
    return out


def expected_exposure(exposures: np.ndarray) -> np.ndarray:
    exposures = np.ascontiguousarray(exposures, dtype=np.float64)
    ee = np.zeros(exposures.shape[1])
    oracle().oracle_expected_exposure(exposures.ravel(), exposures.shape[0], exposures.shape[1], ee)
    return ee


def cva(ee: np.ndarray, n_dates: int, dtau: float, hazard: float, recovery: float) -> tuple[float, float]:
    d = C.c_double(0.0)
    v = oracle().oracle_cva(np.ascontiguousarray(ee, dtype=np.float64), n_dates, dtau, hazard, recovery, C.byref(d))
    return v, d.value


def cva_paths(exposures: np.ndarray, n_dates: int, dtau: float, hazard: float, recovery: float) -> np.ndarray:
    exposures = np.ascontiguousarray(exposures, dtype=np.float64)
    out = np.zeros(exposures.shape[0])
    oracle().oracle_cva_paths(exposures.ravel(), exposures.shape[0], exposures.shape[1], n_dates, dtau, hazard, recovery, out)
    return out


def pfe(exposures: np.ndarray, n_dates: int, q: float) -> np.ndarray:
    exposures = np.ascontiguousarray(exposures, dtype=np.float64)
    out = np.zeros(n_dates)
    oracle().oracle_pfe(exposures.ravel(), exposures.shape[0], exposures.shape[1], n_dates, q, out)
    return out


def trapezoid_drift(vol: np.ndarray, dtau: float) -> np.ndarray:
    vol = np.ascontiguousarray(vol, dtype=np.float64)
    out = np.zeros(vol.shape[1])
    oracle().oracle_trapezoid_drift(vol.ravel(), vol.shape[0], vol.shape[1], dtau, out)
    return out


def philox(ctr, key) -> np.ndarray:
    c = (C.c_uint32 * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    k = (C.c_uint32 * 2)(*[int(x) & 0xFFFFFFFF for x in key])
    o = (C.c_uint32 * 4)()
    oracle().oracle_philox4x32_10(c, k, o)
    return np.array(list(o), dtype=np.uint32)


def host_normals(seed: int, path0: int, n_paths: int, n_steps: int) -> np.ndarray:
    out = np.zeros((n_paths, n_steps, 3))
    oracle().oracle_normals_host(seed, path0, n_paths, n_steps, out.ravel())
    return out


# ---------------------------------------------------------------------------
# cuRAND host generator (no GPU needed)
# ---------------------------------------------------------------------------
CURAND_RNG_PSEUDO_DEFAULT = 100
CURAND_RNG_PSEUDO_PHILOX4_32_10 = 161
_curand = None


def curand_lib():
    global _curand
    if _curand is None:
        cands = []
        cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
        for d in (Path(cuda) / "lib64", Path(cuda) / "targets" / "sbsa-linux" / "lib", Path(cuda) / "targets" / "x86_64-linux" / "lib"):
            cands += sorted(d.glob("libcurand.so*")) if d.exists() else []
        cands.append(Path("libcurand.so.10"))
        last = None
        for c in cands:
            try:
                _curand = C.CDLL(str(c))
                break
            except OSError as e:  # try the next candidate
                last = e
        if _curand is None:
            raise OSError(f"libcurand not found: {last}")
    return _curand


def _gen(kind: int, seed: int):
    lib = curand_lib()
    g = C.c_void_p()
    st = lib.curandCreateGeneratorHost(C.byref(g), C.c_int(kind))
    if st != 0:
        raise RuntimeError(f"curandCreateGeneratorHost failed ({st})")
    st = lib.curandSetPseudoRandomGeneratorSeed(g, C.c_ulonglong(seed))
    if st != 0:
        raise RuntimeError(f"curandSetPseudoRandomGeneratorSeed failed ({st})")
    return lib, g


def curand_normals_double(count: int, seed: int = 1234) -> np.ndarray:
    """The reference's own draws: cuRAND host default (XORWOW) generator,
    curandGenerateNormalDouble(count, 0, 1) (simulation_cpu.h:83-90)."""
    lib, g = _gen(CURAND_RNG_PSEUDO_DEFAULT, seed)
    out = np.zeros(count, dtype=np.float64)
    try:
        st = lib.curandGenerateNormalDouble(g, out.ctypes.data_as(C.c_void_p), C.c_size_t(count), C.c_double(0.0), C.c_double(1.0))
        if st != 0:
            raise RuntimeError(f"curandGenerateNormalDouble failed ({st})")
    finally:
        lib.curandDestroyGenerator(g)
    return out


def curand_philox_u32(count: int, seed: int) -> np.ndarray:
    """cuRAND's host Philox4x32-10 generator.  Its output word 4j+i is word i of
    Philox4x32-10(counter=(0,0,j,0), key=(seed lo, seed hi)) for the first
    blocks, which makes it a known-answer source for our Philox."""
    lib, g = _gen(CURAND_RNG_PSEUDO_PHILOX4_32_10, seed)
    out = np.zeros(count, dtype=np.uint32)
    try:
        st = lib.curandGenerate(g, out.ctypes.data_as(C.c_void_p), C.c_size_t(count))
        if st != 0:
            raise RuntimeError(f"curandGenerate failed ({st})")
    finally:
        lib.curandDestroyGenerator(g)
    return out
