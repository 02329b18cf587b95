"""The C++ drop-in boundary (simulation_gpu.h:12,14) as a C++ caller uses it.

tests/dropin_caller.cpp is compiled with g++ against include/hjm_dropin.h and
libhjmcva.so and calls both calculateExposureMultiGPU overloads the way the
reference's driver does (simulation_gpu_testing.cpp:195-216).  On the CPU:
the caller compiles and links, and so does the reference's own driver,
unchanged, against this library (where the reference tree is present).  On the
GPU: the driver's own workload (its curve, PCA volatility table, drift table
and irregular accruals; N = 10, K = 6.7%, 25y, dt = 0.01) through both
overloads against the oracle on the device's normals (double 1e-10 relative,
float 1e-4), the reference's cuRAND draws through hjm_run_with_normals
against the unmodified reference's EE, and the error behaviour (zero-filled
output, printed note for num_gpus != 1).
"""
from __future__ import annotations

import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle_lib as O
from conftest import load_golden, market_from_golden
from cva_hjm_cuda_gb300 import _lib

ROOT = Path(__file__).resolve().parents[1]
INCLUDE = ROOT / "include"
LIBDIR = _lib.LIB_PATH.parent
CUDA = Path("/usr/local/cuda")

FP64_RTOL = 1e-10
MIXED_RTOL = 1e-4

needs_gxx = pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not found")


def _ensure_lib():
    if not _lib.LIB_PATH.exists():
        from cva_hjm_cuda_gb300 import build

        build.build()


@pytest.fixture(scope="module")
def caller(tmp_path_factory) -> Path:
    """tests/dropin_caller.cpp built against the public headers and the library."""
    if shutil.which("g++") is None:
        pytest.skip("g++ not found")
    _ensure_lib()
    exe = tmp_path_factory.mktemp("dropin") / "dropin_caller"
    subprocess.run(["g++", "-O2", "-std=c++17", "-Wall", "-Werror", f"-I{INCLUDE}", str(ROOT / "tests" / "dropin_caller.cpp"),
                    "-o", str(exe), f"-L{LIBDIR}", "-lhjmcva", f"-Wl,-rpath,{LIBDIR}"], check=True)
    return exe


@needs_gxx
def test_cpp_caller_compiles_and_links(caller):
    assert caller.exists()
    # both overloads resolve to the library's definitions
    out = subprocess.run(["nm", "-u", str(caller)], capture_output=True, text=True).stdout
    assert "_Z25calculateExposureMultiGPUPd16InterestRateSwapIdES_S_S_S_diid" in out
    assert "_Z25calculateExposureMultiGPUPf16InterestRateSwapIfES_S_S_S_fiif" in out


def _reference_tree() -> Path | None:
    try:
        ref = subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "print-ref"], capture_output=True,
                             text=True, check=True).stdout.strip()
    except (OSError, subprocess.CalledProcessError):
        return None
    p = Path(ref)
    return p if (p / "simulation_gpu_testing.cpp").exists() else None


@needs_gxx
def test_reference_driver_compiles_unchanged(tmp_path):
    """The reference's driver (simulation_gpu_testing.cpp, which also constructs an
    InterestRateSwap_D) builds from its own source against include/hjm_dropin.h and links
    against libhjmcva.so in place of the reference's simulation_gpu.cu object.  Its CPU
    path (simulation_cpu.h) needs the MKL stand-in of oracle/shim and cuRAND's host library."""
    ref = _reference_tree()
    if ref is None:
        pytest.skip("reference tree not present")
    _ensure_lib()
    exe = tmp_path / "hjm_driver"
    subprocess.run(["g++", "-O2", "-std=c++17", "-w", f"-I{INCLUDE}", "-include", "hjm_dropin.h",
                    f"-I{ROOT / 'oracle' / 'shim'}", f"-I{CUDA / 'include'}", str(ref / "simulation_gpu_testing.cpp"),
                    "-o", str(exe), f"-L{LIBDIR}", "-lhjmcva", f"-Wl,-rpath,{LIBDIR}", f"-L{CUDA / 'lib64'}",
                    f"-Wl,-rpath,{CUDA / 'lib64'}", "-lcurand"], check=True)
    out = subprocess.run(["nm", "-u", str(exe)], capture_output=True, text=True).stdout
    assert "_Z25calculateExposureMultiGPUPd16InterestRateSwapIdES_S_S_S_diid" in out


# ------------------------------------------------------------------------- GPU
def _write_inputs(path: Path, g: dict) -> None:
    arr = np.concatenate([np.array(g["spot"]), np.array(g["vol"]), np.array(g["drift"]), np.array(g["accrual"]),
                          np.array([g["notional"], g["strike"], g["expiry"], g["dtau"]])])
    arr.astype(np.float64).tofile(path)


def _run_caller(caller: Path, tmp: Path, g: dict, n_paths: int, num_gpus: int = 1, dt: float = 0.01):
    inp, out = tmp / "in.bin", tmp / "out.bin"
    _write_inputs(inp, g)
    r = subprocess.run([str(caller), str(inp), str(out), str(n_paths), str(num_gpus), repr(dt)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    ee = np.fromfile(out, dtype=np.float64)
    return ee[:51], ee[51:], r.stderr


def _as_float_inputs(g: dict) -> dict:
    f = dict(g)
    for k in ("spot", "vol", "drift", "accrual"):
        f[k] = np.array(g[k], dtype=np.float32).astype(np.float64).tolist()
    for k in ("notional", "strike"):
        f[k] = float(np.float32(g[k]))
    return f


def _check(actual, desired, rtol, what):
    actual, desired = np.asarray(actual), np.asarray(desired)
    scale = np.max(np.abs(desired))
    err = np.abs(actual - desired)
    bad = (err > rtol * np.abs(desired)) & (err > rtol * 1e-3 * scale)
    assert not np.any(bad), f"{what}: max rel err {np.max(err / np.maximum(np.abs(desired), 1e-300)):.3e}"


@pytest.mark.gpu
def test_driver_workload_through_both_overloads(engine, caller, tmp_path):
    """The driver's own call (simulation_gpu_testing.cpp:199), both overloads, against the
    oracle on the device's Philox normals (seed 1234, paths 0 .. 4,999, 2,500 steps)."""
    g = load_golden("ref_driver_own_market.json")
    n_paths = 5000
    ee64, ee32, err = _run_caller(caller, tmp_path, g, n_paths)
    assert "ERROR" not in err, err
    normals = engine.dump_normals(n_paths, g["n_steps"], 1234)
    mk, sw = market_from_golden(g)
    ee_orc = O.expected_exposure(O.exposure_paths(mk, sw, g["n_steps"], g["dt"], normals))
    _check(ee64, ee_orc, FP64_RTOL, "double overload vs oracle")
    assert ee64[50] == 0.0 and np.all(ee64[:50] > 0.0)
    gf = _as_float_inputs(g)
    mkf, swf = market_from_golden(gf)
    ee_orc_f = O.expected_exposure(O.exposure_paths(mkf, swf, g["n_steps"], g["dt"], normals))
    _check(ee32, ee_orc_f, MIXED_RTOL, "float overload vs oracle")
    # the two precisions agree with each other as well
    _check(ee32, ee64, MIXED_RTOL, "float vs double overload")


@pytest.mark.gpu
def test_dropin_num_gpus_note_and_zero_fill_on_error(engine, caller, tmp_path):
    g = load_golden("ref_driver_own_market.json")
    ee1, ee1f, _ = _run_caller(caller, tmp_path, g, 256)
    ee4, ee4f, err4 = _run_caller(caller, tmp_path, g, 256, num_gpus=4)
    assert "num_gpus=4" in err4 and "one GPU" in err4
    np.testing.assert_array_equal(ee4, ee1)
    np.testing.assert_array_equal(ee4f, ee1f)
    # dtau / dt = 0.5 / 0.3 is no whole number of steps: printed and zero-filled, as the
    # reference prints and continues (simulation_gpu.cu:71-106); the caller pre-filled NaN
    ee_bad, ee_bad_f, err = _run_caller(caller, tmp_path, g, 256, dt=0.3)
    assert err.count("ERROR") == 2, err
    assert np.all(ee_bad == 0.0) and np.all(ee_bad_f == 0.0)
    # the library's context stays usable after the failed call
    ee_again, _, _ = _run_caller(caller, tmp_path, g, 256)
    np.testing.assert_array_equal(ee_again, ee1)


@pytest.mark.gpu
def test_reference_draws_on_driver_workload(engine):
    """hjm_run_with_normals on the reference's own cuRAND XORWOW draws and the driver's own
    inputs, against the EE of the unmodified calculateExposureCPU<double> and the exposure
    rows of its per-path functions."""
    g = load_golden("ref_driver_own_market.json")
    mk, sw = market_from_golden(g)
    engine.set_market(mk)
    engine.set_swap(sw)
    normals = O.curand_normals_double(g["normals"]["count"], seed=g["normals"]["seed"]).reshape(
        g["n_paths"], g["n_steps"], 3)
    engine.keep_exposures(True)
    try:
        v = engine.run_with_normals(normals, g["n_steps"], g["dt"], "fp64")
        _check(v.ee, g["ee"], FP64_RTOL, "FP64 EE vs reference")
        x = engine.exposures()  # [dates][paths]
        _check(x.T[:16], np.array(g["exposures_first_paths"]), FP64_RTOL, "FP64 exposures vs reference")
    finally:
        engine.keep_exposures(False)
    vm = engine.run_with_normals(normals, g["n_steps"], g["dt"], "mixed")
    _check(vm.ee, g["ee"], MIXED_RTOL, "mixed EE vs reference")
