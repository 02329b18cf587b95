"""CPU checks of bench.py's algorithmic operation counts (the roofline's
numerators): each form's count restated from its kernel's formulas."""
from __future__ import annotations

import bench


def test_response_forms_count_the_kernels_operations():
    nt, n_steps, stride = 51, 1000, 50
    B = n_steps // stride
    # polynomial response form: 9 FMA + 3 ADD per evolved step on the FP64 pipe
    assert bench.algorithmic_flops_per_path(nt, n_steps, stride, "poly_tri", "response") == 21 * (B - 1) * stride
    assert bench.algorithmic_flops_per_path(nt, n_steps, stride, "poly", "response") == 27 * (B - 1) * stride
    # volatility table in the response form: six FMAs per date still to be sampled per step
    live = sum(B - b for b in range(1, B)) * stride
    assert bench.algorithmic_flops_per_path(nt, n_steps, stride, "table", "response") == 12 * live
    # the double-FP32 side: 40 flops per slot, slots in groups of four over the active prefix
    f32 = bench.response_fp32_flops_per_path(nt, n_steps, stride)
    assert f32 % 160 == 0 and 0 < f32 <= 40 * 24 * (B - 1) * stride


def test_convected_forms_exceed_the_response_forms():
    for form in ("poly_tri", "poly", "table"):
        conv = bench.algorithmic_flops_per_path(51, 1000, 50, form)
        resp = bench.algorithmic_flops_per_path(51, 1000, 50, form, "response")
        assert resp < conv, form
