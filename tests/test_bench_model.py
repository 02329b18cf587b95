"""CPU checks of bench.py's algorithmic operation counts (the roofline's
numerators): each form's count restated from its kernel's formulas."""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

import bench

sys.path.insert(0, str(Path(__file__).parent))
import test_cubic_windows as W  # noqa: E402


def test_response_forms_count_the_kernels_operations():
    nt, n_steps, stride = 51, 1000, 50
    B = n_steps // stride
    # polynomial response form: the FP64 pipe forms the parts at the B dates only
    assert bench.algorithmic_flops_per_path(nt, n_steps, stride, "poly_tri", "response") == 41 * B
    assert bench.algorithmic_flops_per_path(nt, n_steps, stride, "poly", "response") == 41 * B
    # volatility table in the response form: no FP64 work per step; on the
    # FP32 pipe three double-FP32 terms (26 flops for both lanes each) and the
    # renormalisation (6) per date still to be sampled per step
    live = sum(B - b for b in range(1, B)) * stride
    assert bench.algorithmic_flops_per_path(nt, n_steps, stride, "table", "response") == 0
    assert bench.table_response_fp32_flops_per_path(nt, n_steps, stride) == (3 * 26 + 6) * live
    # the double-FP32 side: 30 flops per slot (slots in groups of four over the
    # active prefix), 26 per moving-frame term (6 or 9 per step), 18 per step
    # for the renormalisation
    parts_tri = (26 * 6 + 18) * (B - 1) * stride
    f32 = bench.response_fp32_flops_per_path(nt, n_steps, stride) - parts_tri
    assert f32 % 120 == 0 and 0 < f32 <= 30 * 24 * (B - 1) * stride
    assert (bench.response_fp32_flops_per_path(nt, n_steps, stride, "poly")
            - bench.response_fp32_flops_per_path(nt, n_steps, stride, "poly_tri")) == 26 * 3 * (B - 1) * stride


def test_convected_forms_exceed_the_response_forms():
    for form in ("poly_tri", "poly"):
        conv = bench.algorithmic_flops_per_path(51, 1000, 50, form)
        resp = bench.algorithmic_flops_per_path(51, 1000, 50, form, "response")
        assert resp < conv, form


def test_response_slots_follow_the_kernels_value_prefix():
    for nt, n_steps, stride in ((51, 1000, 50), (61, 1000, 50), (51, 600, 25)):
        B = n_steps // stride
        tab, kappa = W.eresp_table(nt, stride, B, 1.0 / stride)
        np.testing.assert_array_equal(bench.response_active_prefix(nt, n_steps, stride),
                                      W.eresp_prefix(tab, kappa, B, stride))


def test_mixed_response_slots_and_count():
    """The mixed-precision response form's slots (mresp_slots restated): the
    10y swap's counting dates fit 8 slots, the 12y swap's 16; the 25y swap on
    51 tenors and the 30y netting shape on 61 tenors convect.  Its count: the
    parts (21 flops per step for factor k of degree <= k) and one packed FMA
    per slot of a date still to be sampled."""
    assert bench.mixed_response_slots(51, 1000, 50) == 8
    assert bench.mixed_response_slots(51, 1200, 50) == 16
    assert bench.mixed_response_slots(51, 2500, 50) == 0
    assert bench.mixed_response_slots(61, 3000, 50) == 0
    # one date: nothing evolves, every slot fits
    assert bench.mixed_response_slots(51, 50, 50) == 8
    B, stride = 20, 50
    want = sum(stride * (21 + 4 * min(8, B - b)) for b in range(1, B))
    assert bench.mixed_response_flops_per_path(51, 1000, 50, "poly_tri") == want
    # far below the convected pairs' count on the same run
    assert want < 0.6 * bench.algorithmic_flops_per_path(51, 1000, 50, "poly_tri")


def test_reference_arm_prints_its_line():
    """bench.py --impl reference (the oracle port on the host cores) runs
    without a GPU and prints one JSON line of the contract."""
    import json
    import subprocess

    root = Path(__file__).resolve().parent.parent
    r = subprocess.run([sys.executable, str(root / "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
