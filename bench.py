#!/usr/bin/env python
"""Benchmark of the HJM exposure / CVA path on one GB300 (path-steps per second).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload fp64|mixed] [--no-extras]

Default workload (``fp64``): the plain FP64 valuation of one payer swap
(notional 1e6, fixed 2.5%, 10y semiannual) on 1,048,576 paths x 1,000 Euler
steps (dt = 0.01) of the 3-factor HJM model on the 51-tenor Nelson-Siegel
curve, with EE, PFE(97.5%) on the 21 reset dates and CVA (hazard 2%,
recovery 40%).  ``mixed``: the same at 4,194,304 paths in mixed precision.
One step = one valuation (path kernel + reductions + PFE selection).  The
timed region holds K steps, each followed by a 256 MiB device write that
evicts L2 (the path kernel reads no input from HBM; its normals are made in
registers).  ``value`` is device-resident throughput (CUDA events on the
launching stream); ``e2e`` repeats the workload through the C ABI call with
host buffers (hjm_run), copies included.  Unless --no-extras, rank 0 also
reports the mixed-precision run against the FP64 run on identical normals,
the measured FMA peaks (roofline denominators) and the CPU baseline (the
oracle port on all host cores, on a bounded sample of the same workload).

``--impl reference`` times the reference algorithm's CPU implementation (the
oracle port, all host threads) on the same workload and prints the same line
with "impl": "reference".  Under torchrun only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "HJM path-steps/s and CVA+deltas time: FP32-mixed vs FP64 on 1 GB300 @1e-4 rel"
UNIT = "path-steps/s"
N_STEPS, DT, SEED = 1000, 0.01, 1234
WORKLOADS = {
    "fp64": {"precision": "fp64", "n_paths": 1_048_576, "dtype": "f64", "n_tenor": 51, "n_steps": 1000,
             "name": "hjm-3f-51tenor-payer-irs-10y-fp64-1048576paths-1000steps"},
    "mixed": {"precision": "mixed", "n_paths": 4_194_304, "dtype": "f32+f64", "n_tenor": 51, "n_steps": 1000,
              "name": "hjm-3f-51tenor-payer-irs-10y-mixed-4194304paths-1000steps"},
    # CVA plus 112 sensitivities by the pathwise adjoint, checkpoints every 32 steps
    "adjoint": {"precision": "mixed", "n_paths": 1_048_576, "dtype": "f32+f64", "n_tenor": 51, "n_steps": 1000,
                "name": "hjm-3f-51tenor-payer-irs-10y-adjoint-ckpt32-1048576paths-1000steps"},
    # 64-swap netting set on a 61-tenor curve, mixed precision
    "netting": {"precision": "mixed", "n_paths": 2_097_152, "dtype": "f32+f64", "n_tenor": 61, "n_steps": 3000,
                "name": "hjm-3f-61tenor-netting64-30y-mixed-2097152paths-3000steps"},
    # the reference driver's own PCA volatility table (cubic factors to its
    # rounding) on the 10y payer swap, FP64
    "reftable": {"precision": "fp64", "n_paths": 1_048_576, "dtype": "f64", "n_tenor": 51, "n_steps": 1000,
                 "market": "reference", "name": "hjm-3f-51tenor-reference-pca-table-irs-10y-fp64-1048576paths"},
    # the reference driver's own workload: its curve, table, drift, accruals,
    # the 25y swap N = 10, K = 6.7% (50 dates), FP64
    "driver25y": {"precision": "fp64", "n_paths": 1_048_576, "dtype": "f64", "n_tenor": 51, "n_steps": 2500,
                  "market": "reference", "swap": "driver",
                  "name": "hjm-3f-51tenor-reference-driver-workload-25y-fp64-1048576paths"},
}
FLUSH_BYTES = 256 << 20


def env_rank():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)),
            int(os.environ.get("WORLD_SIZE", 1)))


def algorithmic_flops_per_path(n_tenor: int, n_steps: int, stride: int, form: str,
                               remainder: str = "convect") -> int:
    """Floating-point operations the path kernel's algorithm needs per path
    (FMA = 2), counted from its formulas, not measured.

    During block b (the steps that end by sampling date b+1) only tenors
    b+1 .. L are ever read again (the upwind step carries information from
    high to low tenors), so the needed convection covers those; in the
    polynomial forms the remainder is also exactly zero below its front
    during the first block.  Per evolved
    Euler step of block b:
    ``poly_tri`` (factor k a polynomial of degree <= k in T, the reference's
    own volatility table): the growth-scaled convection of the remainder
    (L - 1 - b FMAs, 3 FMAs at the last tenor with its source), the scaled
    source coefficient (1 MUL), the updates of the three scalar parts with the
    noise projection folded in (9 FMA), the block sums (3 ADD) and the anchor
    (1 FMA): 2 (NT - b) + 26 flops.  ``poly`` (general quadratic factors): 3
    more FMAs, 2 (NT - b) + 32.
    ``table`` (generic volatility table): 4 FMAs per live tenor (three factor
    loadings and the convection; 5 at the last tenor), the normals' scaling
    (4 MUL), the block sums (3 ADD + 1 FMA): 8 (NT - b) + 3.
    Per block: the block-sum recovery of the tenors still to be sampled
    (about 12 flops each).  The first block holds the curve at spot and does
    no arithmetic.  Normals, pricing and reductions are not counted, and an
    ADD or MUL issues like an FMA, so the fraction is a lower bound on the
    FP64 pipe's use (ncu's pipe utilisation is the direct measure).

    ``remainder="response"`` (FP64): polynomial forms, the FP64 pipe forms the
    parts and their running sums from the moving-frame sums only at the
    sampled dates (41 flops per date: widening the six sums (6), x = M^a y
    (6), Z += Q(a) y - v (15), the two quadratics at the date's tenor (11) and
    the re-anchoring's rests (3)); the per-step work runs in double-FP32 on the
    FP32 pipe (``response_fp32_flops_per_path``); ``table`` (at most 24 dates),
    the same: the whole per-step work in double-FP32 on the FP32 pipe
    (``table_response_fp32_flops_per_path``), nothing per step in FP64."""
    B = n_steps // stride
    L = n_tenor - 1
    if remainder == "response":
        return 41 * B if form != "table" else 0

    def per_step(b: int, k: int) -> int:
        # polynomial forms: the remainder is still zero below tenor L - 1 - k
        # after k evolved steps
        lo = b if form == "table" else max(b, L - 2 - k)
        return {"poly_tri": 2 * (n_tenor - lo) + 26, "poly": 2 * (n_tenor - lo) + 32,
                "table": 8 * (n_tenor - lo) + 3}[form]

    steps = sum(per_step(b, (b - 1) * stride + s) for b in range(1, B) for s in range(stride))
    recovery = 12 * sum(B - b for b in range(1, B))
    return steps + recovery


def response_active_prefix(n_tenor: int, n_steps: int, stride: int, dtau: float = 0.5):
    """Per row b stride + s of the Euler response table, the active prefix the
    kernel reads (eresp_active_kernel, no residual): the slots up to the last
    whose coefficient kappa G_j(lag), in FP32, is nonzero and at least 2^-53
    |kappa|, or whose running-sum coefficient kappa CG_j(lag) is at least
    2^-53 |kappa| j stride; lag = (j - b) stride - 1 - s for date j = B - slot,
    G_j(m) = (A^m e_L)[j] by m upwind steps with c = 1 / stride."""
    import numpy as np

    B, L = n_steps // stride, n_tenor - 1
    c = 1.0 / stride
    kappa = -2.0 * c * dtau * dtau
    rows = B * stride
    width = max(24, B)
    tab = np.zeros((rows, width, 2))
    v = np.zeros(n_tenor)
    v[L] = 1.0
    cum = np.zeros(n_tenor)
    for m in range((B - 1) * stride):
        cum += v
        q = m // stride + 1
        for j in range(max(2, q + 1), B + 1):
            tab[(j - q) * stride + (q * stride - 1 - m), B - j] = (kappa * v[j], kappa * cum[j])
        vn = v.copy()
        vn[:L] = v[:L] + c * (v[1:] - v[:L])
        vn[L] = v[L] + c * (v[L] - v[L - 1])
        v = vn
    a = np.abs(tab.astype(np.float32))
    tg = np.float32(abs(kappa)) * np.float32(2.0 ** -53)
    tcg = (tg * (np.maximum(B - np.arange(width), 1) * stride).astype(np.float32)).astype(np.float32)
    sig = ((a[:, :, 0] != 0) & (a[:, :, 0] >= tg)) | ((a[:, :, 1] != 0) & (a[:, :, 1] >= tcg[None, :]))
    return np.where(sig.any(axis=1), width - np.argmax(sig[:, ::-1], axis=1), 0)


def response_fp32_flops_per_path(n_tenor: int, n_steps: int, stride: int, form: str = "poly_tri") -> int:
    """FP32 flops of the Euler response form's double-FP32 terms per path
    (a multiply or an add 1 flop, an FMA 2; packed instructions count both
    lanes).  At each evolved step: the date slots in groups of four covering
    the row's active prefix (``response_active_prefix``), each slot one packed
    {value, running sum} update of 1 FMUL2 + 3 FFMA2 + 8 FADD2 = 30 flops
    (product with its exact leading term, Knuth two-sum, low-part update); and
    the parts' moving-frame terms, 6 (``poly_tri``) or 9 (``poly``) packed
    {y, v} updates with an exact FP32 normal, 1 FMUL2 + 2 FFMA2 + 8 FADD2 = 26
    flops each, and their renormalisation, 3 x 3 FADD2 = 18 flops.  An add
    occupies the FMA pipe as an FMA does, so the pipe is busier than this
    count's fraction of the FMA peak."""
    B = n_steps // stride
    pre = response_active_prefix(n_tenor, n_steps, stride)[stride:]
    slots = int((4 * ((pre + 3) // 4)).sum())
    terms = 6 if form == "poly_tri" else 9
    return 30 * slots + (26 * terms + 18) * (B - 1) * stride


def table_response_fp32_flops_per_path(n_tenor: int, n_steps: int, stride: int) -> int:
    """FP32 flops per path of the volatility-table step's response form
    (path_kernel_fp64_vresp): per step and date still to be sampled, three
    double-FP32 terms into {value, running sum} (13 flops per lane each: the
    negated product, two FMAs for its error, Knuth's two-sum and the low
    part's update; 26 for the two lanes) and the pairs' renormalisation (3 per
    lane), 84 flops; an add counted as one flop though it occupies the FMA
    pipe like an FMA."""
    B = n_steps // stride
    return 84 * stride * sum(B - b for b in range(1, B))


def mixed_response_slots(n_tenor: int, n_steps: int, stride: int, dtau: float = 0.5) -> int:
    """The date slots of the mixed-precision response form (mresp_slots): 8 or
    16 when every date whose response ever counts (a term kappa G_j(lag) of at
    least 2^-30 |kappa|, or kappa CG_j(lag) of at least 2^-30 |kappa| j stride,
    at the lags date j reads) fits them, else 0 (the run convects)."""
    import numpy as np

    B, L = n_steps // stride, n_tenor - 1
    c = 1.0 / stride
    thr = 2.0 ** -30
    v = np.zeros(n_tenor)
    v[L] = 1.0
    cum = np.zeros(n_tenor)
    need = 0
    j = np.arange(2, B + 1)
    for m in range((B - 1) * stride):
        cum += v
        ok = (m <= (j - 1) * stride - 1) & ((np.abs(v[j]) >= thr) | (np.abs(cum[j]) >= thr * j * stride))
        if ok.any():
            need = max(need, int(B - j[ok].min() + 1))
        vn = v.copy()
        vn[:L] = v[:L] + c * (v[1:] - v[:L])
        vn[L] = v[L] + c * (v[L] - v[L - 1])
        v = vn
    return 8 if need <= 8 else (16 if need <= 16 else 0)


def mixed_response_flops_per_path(n_tenor: int, n_steps: int, stride: int, form: str = "poly_tri") -> int:
    """FP32 flops per path of the mixed-precision response form
    (path_kernel_mixed_resp), counted from its formulas: per evolved step of
    block b, the three scalar parts with the noise projection folded in (9
    FMA for ``poly_tri``, 12 for ``poly``, 15 with the cubic part of
    ``cubic_resid`` and its source), their block sums (3 ADD, 4 with the
    cubic) and, for each slot of a date still to be sampled, one packed FMA
    into {value, running sum} (4 flops).  Normals and pricing are not
    counted."""
    B = n_steps // stride
    ns = mixed_response_slots(n_tenor, n_steps, stride)
    parts = {"poly_tri": 2 * 9 + 3, "poly": 2 * 12 + 3, "cubic_resid": 2 * 16 + 4}[form]
    return sum(stride * (parts + 4 * min(ns, B - b)) for b in range(1, B))


def adjoint_response_flops_per_path(n_tenor: int, n_steps: int, stride: int, form: str = "poly_tri") -> int:
    """FP32 flops per path of the response form's adjoint
    (adjoint_kernel_resp): its forward pass, the mixed response form's count
    (``mixed_response_flops_per_path``), and per reverse step the discount
    seeds into the three moments (3 ADD), the nine coefficient products (9
    FMA), the moments' step (3 FMA + 1 ADD) and one packed FMA (4 flops) per
    slot for the remainder's last-tenor adjoint."""
    B = n_steps // stride
    ns = mixed_response_slots(n_tenor, n_steps, stride)
    reverse = (B - 1) * stride * (3 + 18 + 7 + 4 * ns)
    return mixed_response_flops_per_path(n_tenor, n_steps, stride, form) + reverse


def eresp_windows(n_blocks: int, dates: int = 24) -> list[tuple[int, int]]:
    """The Euler response form's windows of dates, latest first (eresp_windows,
    every date from 2 on active: ``dates`` of them per window)."""
    out, h = [], n_blocks
    while h >= 1:
        lo = h - dates + 1
        if lo <= 2:
            lo = 1
        out.append((lo, h))
        h = lo - 1
    return out


def cubic_fp32_flops_per_path(n_tenor: int, n_steps: int, stride: int, nres: int = 2) -> int:
    """FP32 flops per path of the Euler response form with cubic factors (factor 1
    constant, factors 2 and 3 cubic) and a residual table, counted as
    response_fp32_flops_per_path counts the quadratic form: per window, per
    evolved step up to its last date, each live date slot of the window in
    groups of four (the residual reaches every tenor, so every date still to be
    sampled is active): the residual's packed FMAs (4 flops per residual
    factor) and the renormalisation every fourth step (6 flops / 4), and in the
    groups that reach the remainder's own prefix (``response_active_prefix``;
    the first two groups always) its double-FP32 term (30 flops); the parts'
    moving frame, 9 terms of 26 flops, 4 renormalisations of 6, and the source
    w = y_W + sigma y_X in double-FP32 (14 flops)."""
    B = n_steps // stride
    pre_w = response_active_prefix(n_tenor, n_steps, stride)
    total = 0
    for lo, hi in eresp_windows(B, 16):  # with a residual table the windows hold 16 dates
        roff, nslot = B - hi, hi - max(lo, 2) + 1
        for b in range(1, hi):
            live = sum(1 for j in range(max(lo, 2), hi + 1) if j > b)
            groups = (live + 3) // 4
            for s_ in range(stride):
                n_w = min(max(int(pre_w[b * stride + s_]) - roff, 0), nslot)
                w_groups = min(groups, max(2, (n_w + 3) // 4))
                total += 4 * groups * (4 * nres + 1.5) + 4 * w_groups * 30 + 9 * 26 + 4 * 6 + 14
    return int(total)


class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.proc = None
        self.file = None

    def start(self):
        try:
            self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.file, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().strip().splitlines() if r.count(",") >= 8]
        os.unlink(self.file.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].strip().replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].strip().replace(".", "").isdigit()]
        names = ["active_mask", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i - 4] for r in rows for i in range(5, 9) if r[i].strip().lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def profiled_value(name: str, kernel_key: str) -> float | None:
    """A figure of the dominant kernel from the committed ncu summaries (a line
    ``name[kernel_key]: value``)."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for line in f.read_text().splitlines():
            if line.startswith(f"{name}[{kernel_key}]:"):
                try:
                    return float(line.split(":", 1)[1].strip().split()[0])
                except ValueError:
                    return None
    return None


def profiled_traffic(kernel_key: str) -> float | None:
    """DRAM bytes per launch of the dominant kernel from the committed ncu summaries."""
    return profiled_value("traffic_bytes_per_launch", kernel_key)


def cpu_oracle_sample(target_s: float, n_threads: int) -> dict:
    """The oracle port on all host cores, on a bounded sample of the workload."""
    sys.path.insert(0, str(ROOT / "tests"))
    import numpy as np
    import oracle_lib as O
    from cva_hjm_cuda_gb300.market import Market, Swap

    mk, sw = Market(), Swap()
    lib = O.oracle()
    ee = np.zeros(51)

    def run(n):
        t0 = time.perf_counter()
        rc = lib.oracle_run_mt(51, mk.dtau, DT, N_STEPS, mk.spot, mk.vol.ravel(), mk.drift, sw.accrual, sw.notional,
                               sw.strike, sw.sign, n, SEED, 0, n_threads, ee)
        assert rc == 0
        return time.perf_counter() - t0

    n = 4 * n_threads
    dt = run(n)
    while dt < 0.3:
        n *= 4
        dt = run(n)
    n = max(n_threads, int(n * target_s / dt))
    return {"n_paths": n, "run": run}


def cpu_model() -> str:
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu part", "hardware")):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.processor() or platform.machine()


# ---------------------------------------------------------------------------
def run_reference(args) -> None:
    rank, _, world = env_rank()
    if rank != 0:
        return
    n_threads = os.cpu_count() or 1
    wl = WORKLOADS[args.workload]
    sample = cpu_oracle_sample(target_s=2.0, n_threads=n_threads)
    n = sample["n_paths"]
    for _ in range(args.warmup):
        sample["run"](n)
    times = [sample["run"](n) for _ in range(args.steps)]
    total = sum(times)
    value = n * N_STEPS * args.steps / total
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": wl["name"], "sample_paths_per_step": n, "n_steps": N_STEPS, "dt": DT,
                   "n_tenor": 51, "l2": "n/a (host CPU)"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": n_threads, "kind": "port",
                         "sample": f"{n} paths x {N_STEPS} steps per step (FP64, the workload's first {n} paths)",
                         "cpu": cpu_model()},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import numpy as np
    import torch

    from cva_hjm_cuda_gb300 import HJMEngine, Market, RunConfig, Swap

    rank, local_rank, world = env_rank()
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    wl = WORKLOADS[args.workload]
    n_paths = args.paths or wl["n_paths"]
    prec = wl["precision"]
    n_steps = wl["n_steps"]
    mk, sw = Market(n_tenor=wl["n_tenor"]), Swap(n_tenor=wl["n_tenor"])
    if wl.get("market") == "reference":
        # the reference driver's inputs, from the committed golden fixture
        g = json.loads((ROOT / "tests" / "golden" / "ref_driver_own_market.json").read_text())
        vol = np.array(g["vol"]).reshape(3, 51)
        if wl.get("swap") == "driver":
            mk = Market(n_tenor=51, dtau=0.5, spot=np.array(g["spot"]), vol=vol, drift=np.array(g["drift"]))
            sw = Swap(notional=g["notional"], strike=g["strike"], n_tenor=51, dtau=0.5, accrual=np.array(g["accrual"]))
        else:
            mk = Market(vol=vol)
    stride = int(round(mk.dtau / DT))
    eng = HJMEngine(local_rank)
    # a dedicated (non-default) stream: the engine and the timing events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    eng.set_stream(stream.cuda_stream)
    is_adjoint = args.workload == "adjoint"
    if args.workload == "netting":
        from cva_hjm_cuda_gb300.market import random_netting_set

        netting = random_netting_set(64, seed=20261203)
        set_product = lambda: eng.set_netting_set(netting)  # noqa: E731
    else:
        set_product = lambda: eng.set_swap(sw)  # noqa: E731
    if args.table_step:
        eng.vol_decomposition(False)  # the volatility-table step (profiling)
    if is_adjoint:
        eng.set_market_poly(mk.n_tenor, mk.dtau, mk.spot, mk.vol_coeffs)
    else:
        eng.set_market(mk)
    set_product()
    vol_form = eng.vol_form()
    vol_form_poly = vol_form != "table"
    # weak scaling across ranks: rank r owns paths [r*n, (r+1)*n)
    cfg = RunConfig(n_paths=n_paths, n_steps=n_steps, dt=DT, seed=SEED, path_offset=rank * n_paths)
    flush = torch.empty(FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def one_step():
        if is_adjoint:
            eng.run_adjoint(cfg, checkpoint_every=args.checkpoint_every)  # synchronises: results are copied out
        else:
            eng.enqueue(cfg, prec)

    for _ in range(args.warmup):
        one_step()
        flush.zero_()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = ClockSampler(local_rank)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    launches = 0
    for _ in range(args.steps):
        one_step()
        launches += eng.stats()["kernels"]
        flush.zero_()
    e1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    elapsed = e0.elapsed_time(e1) / 1e3
    if dist:
        t = torch.tensor([elapsed], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t.item())
    value = world * n_paths * n_steps * args.steps / elapsed
    hist = eng.timing_history(min(args.steps, 64))
    path_ms = float(hist[:, 0].mean())
    step_dev_ms = float(hist[:, 3].mean())
    if is_adjoint:
        res = None
    else:
        res = eng.fetch()

    # e2e: the C ABI call with host buffers (market/product arrays in, results
    # out), W untimed calls first as for the device-timed steps (the GPU idles
    # while the clock sampler stops, and the first call after that pays the
    # clock ramp), then K timed calls, each followed by the L2-evicting write
    e2e_times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        if is_adjoint:
            eng.set_market_poly(mk.n_tenor, mk.dtau, mk.spot, mk.vol_coeffs)
            set_product()
            sens = eng.run_adjoint(cfg, checkpoint_every=args.checkpoint_every)
        else:
            eng.set_market(mk)
            set_product()
            eng.run(cfg, prec)
        if i >= args.warmup:
            e2e_times.append(time.perf_counter() - t0)
        flush.zero_()
        torch.cuda.synchronize()
    st = eng.stats()
    h2d = st["h2d_bytes"] + 8 * (mk.spot.size + mk.vol.size + mk.drift.size + sw.accrual.size)
    e2e_value = world * n_paths * n_steps * args.steps / sum(e2e_times)
    # The warm calls above reuse the context's buffers and its cached response
    # table (hjm_set_market with unchanged inputs keeps it).  One cold call: a
    # new context, so its buffers are allocated and the table is built inside
    # the timed call.
    t0 = time.perf_counter()
    with HJMEngine(local_rank) as cold:
        cold.set_stream(stream.cuda_stream)
        if is_adjoint:
            cold.set_market_poly(mk.n_tenor, mk.dtau, mk.spot, mk.vol_coeffs)
        else:
            cold.set_market(mk)
        if args.workload == "netting":
            cold.set_netting_set(netting)
        else:
            cold.set_swap(sw)
        if is_adjoint:
            cold.run_adjoint(cfg, checkpoint_every=args.checkpoint_every)
        else:
            cold.run(cfg, prec)
        cold_s = time.perf_counter() - t0
    torch.cuda.synchronize()

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return

    form = vol_form
    remainder = (("response" if args.checkpoint_every == 0 else "convect") if is_adjoint
                 else eng.remainder_form())
    if is_adjoint and remainder == "response":
        flops = adjoint_response_flops_per_path(mk.n_tenor, n_steps, stride, form) * n_paths
    elif prec != "fp64" and remainder == "response":
        flops = mixed_response_flops_per_path(mk.n_tenor, n_steps, stride, form) * n_paths
    else:
        flops = (algorithmic_flops_per_path(mk.n_tenor, n_steps, stride, form,
                                            "convect" if prec != "fp64" else remainder) * n_paths
                 * (2 if is_adjoint else 1))
    extras = {}
    peak_key = "fp64" if prec == "fp64" else "mixed"
    # the roofline denominators, measured on this GPU (a fraction of a second)
    peak64 = max(eng.fma_peak_tflops("fp64") for _ in range(2))
    peak32 = max(eng.fma_peak_tflops("mixed") for _ in range(2))
    peak = peak64 if peak_key == "fp64" else peak32
    extras["measured_fma_peak_tflops"] = {"fp64": peak64, "fp32": peak32,
                                         "how": "hjm_measure_fma_peak: 8 independent FMA chains per thread, "
                                                "8 CTAs x 256 threads per SM, best of 3 (2 flops per FMA)"}
    achieved = flops / (path_ms * 1e-3) / 1e12
    traffic = profiled_traffic(f"{prec}-table-{n_paths}" if args.table_step else
                               f"{args.workload}-{n_paths}" if wl.get("market") == "reference" else
                               f"{prec}-convect-{n_paths}" if prec != "fp64" and remainder == "convect" else
                               f"{prec}-{n_paths}")
    side = None
    bound = "fp64_pipe" if prec == "fp64" else "fp32_pipe"
    if prec == "fp64" and remainder == "response" and form == "cubic_resid":
        flops = cubic_fp32_flops_per_path(mk.n_tenor, n_steps, stride) * n_paths
        achieved = flops / (path_ms * 1e-3) / 1e12
        peak = extras.get("measured_fma_peak_tflops", {}).get("fp32")
        bound = "fp32_pipe (double-FP32)"
        fma_busy = profiled_value("fma_pipe_cycles_active", f"{args.workload}-{n_paths}")
        side = {"pipe": "fp64 (parts at the sampled dates)", "note": "see the headline workload"}
    elif prec == "fp64" and remainder == "response" and form == "table":
        # the table step's response sums, double-FP32 on the FP32 pipe
        flops = table_response_fp32_flops_per_path(mk.n_tenor, n_steps, stride) * n_paths
        achieved = flops / (path_ms * 1e-3) / 1e12
        peak = extras.get("measured_fma_peak_tflops", {}).get("fp32")
        bound = "fp32_pipe (double-FP32)"
    elif prec == "fp64" and remainder == "response" and form != "table" and not is_adjoint:
        # the per-step work is double-FP32 on the FP32 pipe: that is the
        # roofline; the FP64 pipe only forms the parts at the sampled dates
        side = {"pipe": "fp64 (parts at the sampled dates)", "algorithmic_flops_per_launch": flops,
                "achieved": achieved, "peak": peak, "frac": (achieved / peak) if peak else None}
        flops = response_fp32_flops_per_path(mk.n_tenor, n_steps, stride, form) * n_paths
        achieved = flops / (path_ms * 1e-3) / 1e12
        peak = extras.get("measured_fma_peak_tflops", {}).get("fp32")
        bound = "fp32_pipe (double-FP32)"
        # the FMA pipe's busy fraction from the committed ncu capture: the
        # double-FP32 terms are mostly adds, which occupy it as FMAs do
        fma_busy = profiled_value("fma_pipe_cycles_active", f"{prec}-{n_paths}")
    roofline = {"bound": bound, "achieved": achieved, "peak": peak,
                "unit": "TFLOP/s", "frac": (achieved / peak) if peak else None, "traffic": traffic,
                "kernel": (f"adjoint_kernel_resp<{mixed_response_slots(mk.n_tenor, n_steps, stride)}>"
                           if is_adjoint and remainder == "response" else
                           f"adjoint_kernel<{mk.n_tenor},ckpt,{form}>" if is_adjoint else
                           "path_kernel_fp64_eresp<philox,degs(0,3,3),residual2>"
                           if prec == "fp64" and remainder == "response" and form == "cubic_resid" else
                           f"path_kernel_fp64_vresp<{mk.n_tenor},philox>"
                           if prec == "fp64" and remainder == "response" and form == "table" else
                           "path_kernel_fp64_eresp<philox,degs(0,1,2)>"
                           if prec == "fp64" and remainder == "response" else
                           f"path_kernel_fp64<{mk.n_tenor},philox,{form}>" if prec == "fp64" else
                           f"path_kernel_mixed_resp<philox,{form},{mixed_response_slots(mk.n_tenor, n_steps, stride)}>"
                           if remainder == "response" else
                           f"path_kernel_mixed<{mk.n_tenor},philox,{form}>"),
                "algorithmic_flops_per_launch": flops, "avg_launch_ms": path_ms,
                "peak_source": "measured live by bench.py (FMA microkernel, this GPU)",
                "hbm_peak_gbs_measured": _measured_hbm(),
                # the reference's Euler step, 11 flops per tenor per path-step,
                # at this run's rate (the kernel runs an exact reformulation
                # with far fewer operations; not a roofline of this kernel)
                "reference_equivalent_tflops": 11 * mk.n_tenor * world * n_paths * n_steps * args.steps
                / elapsed / 1e12 if not is_adjoint else None}
    if side:
        roofline["fp64_side"] = side
        roofline["fma_pipe_cycles_active_ncu"] = fma_busy

    if not args.no_extras and prec == "fp64":
        if remainder == "response":
            extras["fp64_convected_form"] = convected_form_run(eng, mk, sw, args, flush, stride, peak64, res)
        extras["generic_table_step"] = generic_step_run(eng, mk, sw, args, flush, stride, peak64, peak32)
        extras["reference_table"] = reference_table_run(eng, args, flush)
        extras["dropin_call"] = dropin_run(args)
        eng.set_market(mk)
        eng.set_swap(sw)
        extras["predictor_corrector"] = predictor_corrector_run(eng, mk, sw, args, flush)
        extras["mlmc"] = mlmc_run(eng, mk, sw)
        extras["mixed"] = mixed_vs_fp64(eng, mk, sw, args, stream, flush, value, peak32)
        extras["adjoint"] = adjoint_cost(eng, args, flush)
        extras["netting"] = netting_set_run(eng, args, flush, peak32)
    if not args.no_extras:
        cb = cpu_oracle_sample(target_s=3.0, n_threads=os.cpu_count() or 1)
        n_cpu = cb["n_paths"]
        t_cpu = cb["run"](n_cpu)
        # the reference's own CPU path is single-threaded: the same port on one thread
        cb1 = cpu_oracle_sample(target_s=1.5, n_threads=1)
        t1 = cb1["run"](cb1["n_paths"])
        cpu_baseline = {"value": n_cpu * N_STEPS / t_cpu, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                        "sample": f"first {n_cpu} paths x {N_STEPS} steps, FP64, oracle port, all host threads",
                        "cpu": cpu_model(),
                        "single_thread": {"value": cb1["n_paths"] * N_STEPS / t1, "unit": UNIT, "cores": 1,
                                          "sample": f"first {cb1['n_paths']} paths x {N_STEPS} steps"}}
    else:
        cpu_baseline = None

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": wl["dtype"], "data": "synthetic",
        "config": {"workload": (wl["name"].replace("ckpt32", f"ckpt{args.checkpoint_every}"
                                                   if args.checkpoint_every else "sampled-states")
                                if is_adjoint else wl["name"]), "n_paths_per_gpu": n_paths, "n_steps": n_steps, "dt": DT,
                   "n_tenor": mk.n_tenor, "factors": 3, "sampled_dates": n_steps // stride,
                   "pfe_quantile": None if is_adjoint else 0.975, "hazard": 0.02,
                   "recovery": 0.4, "seed": SEED,
                   "vol_form": ("cubic factors with a residual table (the reference driver's PCA table): "
                                "decomposed step" if vol_form == "cubic_resid" else
                                "quadratic factors (detected in the volatility table): decomposed step" if vol_form_poly
                                else "volatility table: generic step"),
                   "remainder": remainder,
                   "arithmetic": (("FP64 deterministic curve, parts at the sampled dates, pricing, discounting "
                                   "and reductions; per step the stochastic parts S, U, W (moving frame) and the "
                                   "remainder's response sums in double-FP32 (48-bit) on the FP32 pipe: a path's "
                                   "exposures within ~2e-13 of the exposure scale of the all-FP64 step "
                                   "(fp64_convected_form), EE and CVA within 1e-10 of the FP64 oracle"
                                   if form != "table" else
                                   "FP64 deterministic curve, pricing, discounting and reductions; per step the "
                                   "three factors' impulse-response sums (value and running sum per date) in "
                                   "double-FP32 (48-bit) on the FP32 pipe")
                                  if remainder == "response" and prec == "fp64" else None),
                   "path_step": ("one Euler step of one path's whole tenor curve, the reference's unit; the "
                                 "response form computes the same values by exact algebra without evolving every "
                                 "tenor (fp64_convected_form times the curve-evolving FP64 kernel on the same "
                                 "paths)"),
                   "parallelism": f"replicas{world}" if world > 1 else "single",
                   "l2": f"flushed between steps ({FLUSH_BYTES >> 20} MiB device write, inside the timed region)"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(st["d2h_bytes"]), "call": "hjm_set_market + hjm_set_swap + hjm_run",
                "plan": "warm: the context's buffers and response table (a plan cached per run shape and "
                        "market) are reused across calls",
                "ms_per_call": {"median": 1e3 * statistics.median(e2e_times), "min": 1e3 * min(e2e_times),
                                "max": 1e3 * max(e2e_times), "warmup_calls": args.warmup},
                "cold_call": {"value": world * n_paths * n_steps / cold_s, "unit": UNIT, "ms": 1e3 * cold_s,
                              "what": "one call on a new context: device buffers allocated and the response "
                                      "table built inside the timed call"}},
        "gpu_launches": launches,
        "roofline": roofline,
        "cpu_baseline": cpu_baseline,
        "clocks": clk,
        "device_ms_per_step": step_dev_ms,
        "result": ({"cva": sens.cva, "cva_stderr": sens.cva_stderr, "dcva_dhazard": sens.dcva_dhazard}
                   if is_adjoint else
                   {"cva": res.cva, "cva_stderr": res.cva_stderr, "ee_0": float(res.ee[0]),
                    "pfe_0": float(res.pfe[0]) if res.pfe is not None else None}),
    }
    line.update(extras)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def fp32_roofline(kernel: str, flops_per_launch: float, launch_ms: float, peak32: float | None,
                  traffic_key: str) -> dict:
    """The roofline block of an FP32-pipe kernel (mixed precision): algorithmic
    flops per launch (``algorithmic_flops_per_path``) over the average launch
    time, against the measured FP32 FMA peak; DRAM traffic per launch from the
    committed ncu summary."""
    achieved = flops_per_launch / (launch_ms * 1e-3) / 1e12
    out = {"bound": "fp32_pipe", "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
           "frac": (achieved / peak32) if peak32 else None, "traffic": profiled_traffic(traffic_key),
           "kernel": kernel, "algorithmic_flops_per_launch": flops_per_launch, "avg_launch_ms": launch_ms,
           "peak_source": "measured live by bench.py (FMA microkernel, this GPU)"}
    # the busiest pipe's share from the committed ncu capture, where one is
    # recorded (the generator's integer multiplies share it with the FMAs)
    busy = profiled_value("fmaheavy_pipe_cycles_active", traffic_key)
    if busy is not None:
        out["fmaheavy_pipe_cycles_active_ncu"] = busy
    return out


def _measured_hbm():
    f = ROOT / "MEASURED_PEAKS.json"
    try:
        return json.loads(f.read_text()).get("hbm_gbs")
    except (OSError, ValueError):
        return None


def reference_table_run(eng, args, flush) -> dict:
    """The reference driver's own volatility table (simulation_gpu_testing.cpp:47-63,
    cubic factors to its 9-decimal rounding, read from the committed golden fixture)
    in FP64 on 1,048,576 paths: the 10y payer swap of the headline (20 dates, one
    window) and the driver's own 25y swap (N = 10, K = 6.7%, its accruals and
    spot curve; 50 dates, three windows), each in the cubic response form and in
    the convected table step on the same paths."""
    import numpy as np
    import torch

    from cva_hjm_cuda_gb300 import RunConfig
    from cva_hjm_cuda_gb300.market import Market, Swap

    g = json.loads((ROOT / "tests" / "golden" / "ref_driver_own_market.json").read_text())
    vol = np.array(g["vol"]).reshape(3, 51)
    own = Market(n_tenor=51, dtau=0.5, spot=np.array(g["spot"]), vol=vol, drift=np.array(g["drift"]))
    drv = Swap(notional=g["notional"], strike=g["strike"], n_tenor=51, dtau=0.5, accrual=np.array(g["accrual"]))
    n = WORKLOADS["fp64"]["n_paths"]
    out = {}
    for label, mk, sw, n_steps in (("10y_swap", Market(vol=vol), Swap(), 1000), ("driver_25y_swap", own, drv, 2500)):
        eng.set_market(mk)
        eng.set_swap(sw)
        cfg = RunConfig(n_paths=n, n_steps=n_steps, dt=DT, seed=SEED)
        res = {"n_paths": n, "n_steps": n_steps, "dates": n_steps // 50, "vol_form": eng.vol_form()}
        for form, steps in (("auto", args.steps), ("convect", 2)):
            eng.set_remainder_form(form)
            for _ in range(2 if form == "convect" else args.warmup):
                eng.enqueue(cfg, "fp64", pfe=False)
                flush.zero_()
            torch.cuda.synchronize()
            for _ in range(steps):
                eng.enqueue(cfg, "fp64", pfe=False)
                flush.zero_()
            torch.cuda.synchronize()
            hist = eng.timing_history(steps)
            r = eng.fetch()
            key = "response_form" if form == "auto" else "convected_table_step"
            res[key] = {"remainder": eng.remainder_form(), "path_kernel_ms": float(hist[:, 0].mean()),
                        "device_ms_per_step": float(hist[:, 3].mean()),
                        "path_steps_per_s": n * n_steps / (float(hist[:, 3].mean()) * 1e-3), "cva": r.cva,
                        "ee": [float(x) for x in r.ee[: n_steps // 50]]}
        eng.set_remainder_form("auto")
        a, b = np.array(res["response_form"]["ee"]), np.array(res["convected_table_step"]["ee"])
        res["ee_max_rel_diff"] = float(np.max(np.abs(a - b) / np.abs(b)))
        res["speedup"] = res["response_form"]["path_steps_per_s"] / res["convected_table_step"]["path_steps_per_s"]
        out[label] = res
    return out


def dropin_run(args) -> dict:
    """The reference's own entry point, calculateExposureMultiGPU (double
    overload, simulation_gpu.h:12; the float overload, :14, on the driver's
    call as well), through the C++ drop-in of the library:
    host arrays in, the 51-point EE out, timed end to end on the host (the
    drop-in's process-wide context is warm after the first call).  On the
    headline market and swap (1,048,576 paths, 10y) and on the reference
    driver's own call (its curve, PCA table, drift, accruals, N = 10, K = 6.7%,
    25y; 1,048,576 paths instead of the driver's default 100,000)."""
    import numpy as np

    from cva_hjm_cuda_gb300.engine import calculate_exposure_gpu, calculate_exposure_gpu_fp32
    from cva_hjm_cuda_gb300.market import Market, Swap

    g = json.loads((ROOT / "tests" / "golden" / "ref_driver_own_market.json").read_text())
    mk, sw = Market(), Swap()
    cases = {
        "headline_10y": (sw.notional, sw.strike, 10.0, sw.accrual, mk.spot, mk.drift, mk.vol.ravel()),
        "reference_driver_25y": (g["notional"], g["strike"], g["expiry"], np.array(g["accrual"]), np.array(g["spot"]),
                                 np.array(g["drift"]), np.array(g["vol"])),
    }
    out = {}
    n = WORKLOADS["fp64"]["n_paths"]
    for label, (notional, strike, expiry, acc, spot, drift, vol) in cases.items():
        ee = np.zeros(51)
        steps = int(round(expiry / DT))
        for _ in range(args.warmup):
            calculate_exposure_gpu(ee, notional, strike, expiry, 0.5, acc, spot, drift, vol, 0.0, 1, n, DT)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            calculate_exposure_gpu(ee, notional, strike, expiry, 0.5, acc, spot, drift, vol, 0.0, 1, n, DT)
            times.append(time.perf_counter() - t0)
        t = statistics.median(times)
        out[label] = {"n_paths": n, "n_steps": steps, "ms_per_call": 1e3 * t, "path_steps_per_s": n * steps / t,
                      "ee_0": float(ee[0])}
    # the float overload (simulation_gpu.h:14: the library's mixed precision)
    # on the reference driver's own call, the same paths
    notional, strike, expiry, acc, spot, drift, vol = cases["reference_driver_25y"]
    ee32 = np.zeros(51, dtype=np.float32)
    steps = int(round(expiry / DT))
    for _ in range(args.warmup):
        calculate_exposure_gpu_fp32(ee32, notional, strike, expiry, 0.5, acc, spot, drift, vol, 0.0, 1, n, DT)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        calculate_exposure_gpu_fp32(ee32, notional, strike, expiry, 0.5, acc, spot, drift, vol, 0.0, 1, n, DT)
        times.append(time.perf_counter() - t0)
    t = statistics.median(times)
    ee64 = out["reference_driver_25y"]["ee_0"]
    out["reference_driver_25y_float"] = {"n_paths": n, "n_steps": steps, "ms_per_call": 1e3 * t,
                                         "path_steps_per_s": n * steps / t, "ee_0": float(ee32[0]),
                                         "ee_0_rel_diff_vs_double_overload": abs(float(ee32[0]) - ee64) / abs(ee64)}
    return out


def mixed_vs_fp64(eng, mk, sw, args, stream, flush, fp64_value, peak32=None) -> dict:
    """Mixed precision at 4,194,304 paths: throughput, and its error against the
    FP64 valuation of the same paths (identical normals)."""
    import numpy as np
    import torch

    from cva_hjm_cuda_gb300 import RunConfig

    n = WORKLOADS["mixed"]["n_paths"]
    cfg = RunConfig(n_paths=n, n_steps=N_STEPS, dt=DT, seed=SEED)
    for _ in range(args.warmup):
        eng.enqueue(cfg, "mixed")
        flush.zero_()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        eng.enqueue(cfg, "mixed")
        flush.zero_()
    e1.record(stream)
    torch.cuda.synchronize()
    el = e0.elapsed_time(e1) / 1e3
    hist = eng.timing_history(min(args.steps, 64))
    mx = eng.fetch()
    mx_form = eng.remainder_form()
    f64 = eng.run(cfg, "fp64")
    f64_ms = float(eng.timing_history(1)[0, 0])
    rel = np.abs(mx.ee[:20] - f64.ee[:20]) / f64.ee[:20]
    value = n * N_STEPS * args.steps / el
    stride = int(round(mk.dtau / DT))
    kern_ms = float(hist[:, 0].mean())
    form = eng.vol_form()
    engine_form = mx_form
    if engine_form == "response":
        flops = mixed_response_flops_per_path(mk.n_tenor, N_STEPS, stride, form) * n
        kname = f"path_kernel_mixed_resp<philox,{form},{mixed_response_slots(mk.n_tenor, N_STEPS, stride)}>"
    else:
        flops = algorithmic_flops_per_path(mk.n_tenor, N_STEPS, stride, form, "convect") * n
        kname = f"path_kernel_mixed<{mk.n_tenor},philox,{form}>"
    return {
        "value": value, "unit": UNIT, "n_paths": n, "ms_per_step": 1e3 * el / args.steps,
        "path_kernel_ms": kern_ms, "remainder": engine_form,
        "roofline": fp32_roofline(kname, flops, kern_ms, peak32,
                                  f"mixed-{n}" if engine_form == "response" else f"mixed-convect-{n}"),
        "speedup_vs_fp64_path_steps_per_s": value / fp64_value,
        "fp64_same_paths_path_kernel_ms": f64_ms,
        "ee_rel_err_vs_fp64_per_date": [float(x) for x in rel],
        "ee_max_rel_err_vs_fp64": float(rel.max()),
        "cva": mx.cva, "cva_fp64": f64.cva, "cva_rel_err_vs_fp64": abs(mx.cva - f64.cva) / f64.cva,
        "cva_stderr": mx.cva_stderr,
        "pfe_max_rel_err_vs_fp64": float(np.max(np.abs(mx.pfe[:20] - f64.pfe[:20]) / f64.pfe[:20])),
    }


def generic_step_run(eng, mk, sw, args, flush, stride, peak64, peak32) -> dict:
    """The same valuations with the polynomial decomposition switched off (the
    generic volatility-table step every market can use)."""
    import torch

    from cva_hjm_cuda_gb300 import RunConfig

    out = {}
    eng.vol_decomposition(False)
    try:
        eng.set_market(mk)
        eng.set_swap(sw)
        for prec, n, peak in (("fp64", WORKLOADS["fp64"]["n_paths"], peak64),
                              ("mixed", WORKLOADS["mixed"]["n_paths"], peak32)):
            cfg = RunConfig(n_paths=n, n_steps=N_STEPS, dt=DT, seed=SEED)
            for _ in range(args.warmup):
                eng.enqueue(cfg, prec)
                flush.zero_()
            torch.cuda.synchronize()
            for _ in range(args.steps):
                eng.enqueue(cfg, prec)
                flush.zero_()
            torch.cuda.synchronize()
            hist = eng.timing_history(min(args.steps, 64))
            kern_ms, step_ms = float(hist[:, 0].mean()), float(hist[:, 3].mean())
            res = eng.fetch()
            form = eng.remainder_form() if prec == "fp64" else "convect"
            fl = algorithmic_flops_per_path(mk.n_tenor, N_STEPS, stride, "table", form) * n
            if form == "response":  # the double-FP32 response sums, on the FP32 pipe
                fl, peak = table_response_fp32_flops_per_path(mk.n_tenor, N_STEPS, stride) * n, peak32
            out[prec] = {"n_paths": n, "remainder": form,
                         "path_steps_per_s": n * N_STEPS / (step_ms * 1e-3), "device_ms_per_step": step_ms,
                         "path_kernel_ms": kern_ms, "achieved_tflops": fl / (kern_ms * 1e-3) / 1e12,
                         "frac_of_measured_fma_peak": (fl / (kern_ms * 1e-3) / 1e12 / peak) if peak else None,
                         "cva": res.cva}
    finally:
        eng.vol_decomposition(True)
        eng.set_market(mk)
        eng.set_swap(sw)
    return out


def convected_form_run(eng, mk, sw, args, flush, stride, peak64, res_resp) -> dict:
    """The headline valuation with the decomposition's remainder convected in
    FP64 over the live tenors (every operation of the curve in FP64), against
    the response form's run on the same paths."""
    import numpy as np
    import torch

    from cva_hjm_cuda_gb300 import RunConfig

    n = WORKLOADS["fp64"]["n_paths"]
    cfg = RunConfig(n_paths=n, n_steps=N_STEPS, dt=DT, seed=SEED)
    eng.set_remainder_form("convect")
    try:
        for _ in range(args.warmup):
            eng.enqueue(cfg, "fp64")
            flush.zero_()
        torch.cuda.synchronize()
        for _ in range(args.steps):
            eng.enqueue(cfg, "fp64")
            flush.zero_()
        torch.cuda.synchronize()
        hist = eng.timing_history(min(args.steps, 64))
        kern_ms, step_ms = float(hist[:, 0].mean()), float(hist[:, 3].mean())
        res = eng.fetch()
        assert eng.remainder_form() == "convect"
    finally:
        eng.set_remainder_form("auto")
    fl = algorithmic_flops_per_path(mk.n_tenor, N_STEPS, stride, eng.vol_form()) * n
    return {"n_paths": n, "path_steps_per_s": n * N_STEPS / (step_ms * 1e-3), "device_ms_per_step": step_ms,
            "path_kernel_ms": kern_ms, "achieved_tflops": fl / (kern_ms * 1e-3) / 1e12,
            "frac_of_measured_fma_peak": (fl / (kern_ms * 1e-3) / 1e12 / peak64) if peak64 else None,
            "cva": res.cva, "response_form_cva": res_resp.cva,
            "ee_max_rel_diff_vs_response_form": float(np.max(np.abs(res.ee[1:20] - res_resp.ee[1:20])
                                                             / np.abs(res_resp.ee[1:20])))}


def predictor_corrector_run(eng, mk, sw, args, flush) -> dict:
    """The valuations under the predictor-corrector scheme (three-point
    convection, table volatility step), and their EE difference from Euler."""
    import numpy as np
    import torch

    from cva_hjm_cuda_gb300 import RunConfig

    out = {}
    eng.set_market(mk)
    eng.set_swap(sw)
    try:
        for prec, n in (("fp64", WORKLOADS["fp64"]["n_paths"]), ("mixed", WORKLOADS["mixed"]["n_paths"])):
            cfg = RunConfig(n_paths=n, n_steps=N_STEPS, dt=DT, seed=SEED)
            eng.set_scheme("euler")
            eu = eng.run(cfg, prec)
            eng.set_scheme("predictor_corrector")
            for _ in range(args.warmup):
                eng.enqueue(cfg, prec)
                flush.zero_()
            torch.cuda.synchronize()
            for _ in range(args.steps):
                eng.enqueue(cfg, prec)
                flush.zero_()
            torch.cuda.synchronize()
            hist = eng.timing_history(min(args.steps, 64))
            step_ms = float(hist[:, 3].mean())
            res = eng.fetch()
            out[prec] = {"n_paths": n, "path_steps_per_s": n * N_STEPS / (step_ms * 1e-3),
                         "device_ms_per_step": step_ms, "path_kernel_ms": float(hist[:, 0].mean()),
                         "cva": res.cva, "cva_euler": eu.cva,
                         "ee_max_rel_diff_vs_euler": float(np.max(np.abs(res.ee[:20] - eu.ee[:20]) / eu.ee[:20]))}
        # the adjoint under the scheme (mixed precision, the sampled states kept)
        # against one mixed-precision valuation of the same paths
        n = WORKLOADS["adjoint"]["n_paths"]
        cfg = RunConfig(n_paths=n, n_steps=N_STEPS, dt=DT, seed=SEED)
        eng.set_market_poly(mk.n_tenor, mk.dtau, mk.spot, mk.vol_coeffs)
        eng.set_swap(sw)
        for _ in range(args.warmup):
            eng.run_adjoint(cfg, checkpoint_every=0)
        adj_ms = []
        for _ in range(args.steps):
            eng.run_adjoint(cfg, checkpoint_every=0)
            adj_ms.append(float(eng.timing_history(1)[0, 0]))
        for _ in range(args.warmup):
            eng.enqueue(cfg, "mixed", pfe=False)
        torch.cuda.synchronize()
        for _ in range(args.steps):
            eng.enqueue(cfg, "mixed", pfe=False)
        torch.cuda.synchronize()
        val_ms = float(eng.timing_history(min(args.steps, 64))[:, 0].mean())
        out["adjoint"] = {"n_paths": n, "checkpoint_every": 0, "adjoint_ms": float(np.mean(adj_ms)),
                          "one_cva_valuation_ms": val_ms, "adjoint_cost_in_valuations": float(np.mean(adj_ms)) / val_ms}
    finally:
        eng.set_scheme("euler")
        eng.set_market(mk)
        eng.set_swap(sw)
    return out


def mlmc_run(eng, mk, sw) -> dict:
    """Multi-level Monte Carlo against a plain valuation on the finest grid
    (dt = 0.00625, 1,600 steps for the 10y swap; levels dt = 0.1 / 2^l, l =
    0..4), both in mixed precision at the same CVA standard error: a pilot
    run gives each level's per-path variance and cost, the Giles allocation
    the paths per level."""
    import numpy as np

    from cva_hjm_cuda_gb300 import RunConfig
    from cva_hjm_cuda_gb300.engine import mlmc_allocation

    eng.set_market(mk)
    eng.set_swap(sw)
    n_plain = WORKLOADS["fp64"]["n_paths"]
    fine = RunConfig(n_paths=n_plain, n_steps=1600, dt=0.00625, seed=SEED)
    eng.run(fine, "mixed", pfe=False)  # warm-up
    plain = eng.run(fine, "mixed", pfe=False)
    plain_ms = float(eng.timing_history(1)[0, 3])
    levels = 5
    pilot = eng.run_mlmc([65536] * levels, n_steps=100, dt=0.1, seed=SEED + 1)
    var = [lv["stderr"] ** 2 * lv["n_paths"] for lv in pilot["levels"]]
    cost = [lv["ms"] / lv["n_paths"] for lv in pilot["levels"]]
    n = mlmc_allocation(var, cost, plain.cva_stderr)
    m = eng.run_mlmc(list(n), n_steps=100, dt=0.1, seed=SEED + 2)
    ms = sum(lv["ms"] for lv in m["levels"])
    return {"finest_dt": 0.00625, "levels": levels, "plain_paths": n_plain, "plain_ms": plain_ms,
            "plain_cva": plain.cva, "plain_stderr": plain.cva_stderr, "mlmc_paths_per_level": [int(x) for x in n],
            "mlmc_ms": ms, "mlmc_cva": m["cva"], "mlmc_stderr": m["cva_stderr"],
            "speedup_at_equal_stderr": plain_ms / ms,
            "level_var_per_path": [float(v) for v in var], "level_cost_ms_per_path": [float(c) for c in cost]}


def adjoint_cost(eng, args, flush) -> dict:
    """Config 4: CVA plus its sensitivities to the 51 initial forwards, the drift
    table, the 9 volatility coefficients and the hazard rate, by the pathwise
    adjoint (1,048,576 paths, FP32 forward with FP64 accumulators, checkpoints
    every 32 steps), against one CVA valuation of the same paths."""
    import numpy as np
    import torch

    from cva_hjm_cuda_gb300 import RunConfig
    from cva_hjm_cuda_gb300.market import DEFAULT_VOL_COEFFS, Swap, nelson_siegel_curve, tenor_grid

    n = 1_048_576
    eng.set_market_poly(51, 0.5, nelson_siegel_curve(tenor_grid(51, 0.5)), DEFAULT_VOL_COEFFS)
    eng.set_swap(Swap())
    cfg = RunConfig(n_paths=n, n_steps=N_STEPS, dt=DT, seed=SEED)
    out = {"n_paths": n, "n_sensitivities": 51 + 51 + 9 + 1}
    # checkpoints every 32 steps: the convected adjoint (curve states stored
    # and recomputed); none: the response form's adjoint, which keeps each
    # date's sampled state (the sweep needs no other forward state)
    for label, k in (("checkpoint_32", 32), ("no_checkpoint", 0)):
        for _ in range(args.warmup):
            eng.run_adjoint(cfg, checkpoint_every=k)
        ms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            sens = eng.run_adjoint(cfg, checkpoint_every=k)
            ms.append(float(eng.timing_history(1)[0, 3]))
        out[label] = {"ms": statistics.median(ms), "remainder": "convect" if k else "response"}
    for _ in range(args.warmup):
        eng.run(cfg, "mixed", pfe=False)
    ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        v = eng.run(cfg, "mixed", pfe=False)
        ms.append(float(eng.timing_history(1)[0, 3]))
    one = statistics.median(ms)
    out["one_cva_valuation_ms"] = one
    out["one_cva_valuation_remainder"] = eng.remainder_form()
    # the adjoint's forward pass convects the remainder: the valuation in that
    # form as well (the default valuation carries it in FP32 responses)
    eng.set_remainder_form("convect")
    try:
        for _ in range(args.warmup):
            eng.run(cfg, "mixed", pfe=False)
        ms = []
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            eng.run(cfg, "mixed", pfe=False)
            ms.append(float(eng.timing_history(1)[0, 3]))
    finally:
        eng.set_remainder_form("auto")
    conv = statistics.median(ms)
    out["one_cva_valuation_convected_ms"] = conv
    for label in ("checkpoint_32", "no_checkpoint"):
        out[label]["cost_in_valuations"] = out[label]["ms"] / one
        out[label]["cost_in_convected_valuations"] = out[label]["ms"] / conv
    # one-sided bump-and-revalue of the 51 forwards, 9 coefficients and the hazard
    out["bump_and_revalue_valuations"] = 1 + 51 + 9 + 1
    out["cva"] = sens.cva
    out["cva_same_paths_forward"] = v.cva
    out["dcva_dspot_sum"] = float(np.sum(sens.dcva_dspot))
    out["dcva_dhazard"] = sens.dcva_dhazard
    return out


def netting_set_run(eng, args, flush, peak32=None) -> dict:
    """Config 5: 64 payer/receiver swaps (maturities 1-30y) on a 61-tenor curve,
    3,000 steps, 2,097,152 paths, mixed precision: the netted EE/PFE/CVA
    valuation and the adjoint, each one fused launch (plus reductions)."""
    import numpy as np
    import torch

    from cva_hjm_cuda_gb300 import RunConfig
    from cva_hjm_cuda_gb300.market import DEFAULT_VOL_COEFFS, nelson_siegel_curve, random_netting_set, tenor_grid

    n, steps = 2_097_152, 3000
    ns = random_netting_set(64, seed=20261203)
    eng.set_market_poly(61, 0.5, nelson_siegel_curve(tenor_grid(61, 0.5)), DEFAULT_VOL_COEFFS)
    eng.set_netting_set(ns)
    cfg = RunConfig(n_paths=n, n_steps=steps, dt=DT, seed=SEED)
    for _ in range(args.warmup):
        eng.enqueue(cfg, "mixed")
    torch.cuda.synchronize()
    for _ in range(args.steps):
        eng.enqueue(cfg, "mixed")
    v = eng.fetch()
    hist = eng.timing_history(min(args.steps, 64))
    val_ms = float(np.median(hist[:, 3]))
    eng.run_adjoint(cfg, checkpoint_every=32)
    ms = []
    for _ in range(max(1, args.steps // 2)):
        flush.zero_()
        torch.cuda.synchronize()
        sens = eng.run_adjoint(cfg, checkpoint_every=32)
        ms.append(float(eng.timing_history(1)[0, 3]))
    adj_ms = statistics.median(ms)
    kern_ms = float(np.median(hist[:, 0]))
    flops = algorithmic_flops_per_path(61, steps, 50, "poly_tri", "convect") * n
    return {"n_paths": n, "n_steps": steps, "n_tenor": 61, "n_swaps": len(ns), "dates": steps // 50,
            "valuation_ms": val_ms, "path_steps_per_s": n * steps / (val_ms * 1e-3),
            "path_kernel_ms": kern_ms,
            "roofline": fp32_roofline("path_kernel_mixed<61,philox,poly_tri,compact>", flops, kern_ms, peak32,
                                      f"mixed-{n}"),
            "cva": v.cva, "cva_stderr": v.cva_stderr,
            "adjoint_ms_checkpoint_32": adj_ms, "adjoint_cost_in_valuations": adj_ms / val_ms,
            "adjoint_cva": sens.cva}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="fp64")
    ap.add_argument("--paths", type=int, default=0, help="override the workload's path count (profiling only)")
    ap.add_argument("--checkpoint-every", type=int, default=32,
                    help="adjoint workload: curve checkpoints every K steps (0: the sampled states kept, "
                         "the response form's adjoint)")
    ap.add_argument("--no-extras", action="store_true", help="only the headline workload")
    ap.add_argument("--table-step", action="store_true",
                    help="run the workload on the volatility-table step (no decomposition; profiling only)")
    args = ap.parse_args()
    if args.warmup < 3:
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
