"""Canonical algorithmic work counts of the hot-path kernels (one source of truth).

Per kernel evaluation (one test point x one source point):

* MoM CFIE (the reference's EFIE + MFIE integrand, per-test-point moment form
  sum_j G, sum_j G y_j, sum_j h, sum_j h y_j):           50 FP32 FLOP, 3 MUFU (rsqrt, sin, cos)
* MoM EFIE only:                                       30 FP32 FLOP, 3 MUFU
* Laplace single layer (1/4 pi R times P1 products):   15 FP32 FLOP, 1 MUFU (rsqrt)
* Laplace double layer (grad_y G . n times P1):        22 FP32 FLOP, 1 MUFU
* Scattered H per (field point, vertex) pair ((1 + jkR) e^{jkR} / (4 pi R^3) times the
  complex cross product (A J) x (x - y), accumulated):   61 FP32 FLOP, 3 MUFU (rsqrt, sin, cos)

An FMA counts as 2 FLOP.  Units: a "triangle pair" is one ordered (test, source) face
pair; with the reference's collapsed Gauss rule of order q (test q^2 points, source
(q-1)^2 points, rotated per local edge) a pair costs 9 * q^2 * (q-1)^2 evaluations.
Matrix-vector products are HBM-bound: 8 E^2 + 16 E bytes per complex64 matvec.
"""
from __future__ import annotations

import json
import os

CFIE_FLOP_PER_EVAL = 50
CFIE_MUFU_PER_EVAL = 3
EFIE_FLOP_PER_EVAL = 30
EFIE_MUFU_PER_EVAL = 3
LAPLACE_SL_FLOP_PER_EVAL = 15
LAPLACE_DL_FLOP_PER_EVAL = 22
LAPLACE_MUFU_PER_EVAL = 1
# symmetric-rule P1 single layer (7 x 7 points per separated face pair): per evaluation
# 3 (x - y) + 5 (|d|^2) + 1 (w / R) + 6 (three hat-weighted sums) FLOP and one rsqrt; per
# outer point 15 (the point) + 1 (weight) + 21 (the 3 x 3 block) FLOP, ~5 per evaluation
LAPLACE_SYM_P1_FLOP_PER_EVAL = 20
RADIATE_FLOP_PER_PAIR = 61
RADIATE_MUFU_PER_PAIR = 3
# nominal FP64 rate of a GB300 (far below its FP32 SIMT rate); used only as the denominator
# of FP64 kernels, which have no measured figure
FP64_NOMINAL_TFLOPS = 1.25

GB300_SMS = 152  # only used when no CUDA device can be queried (CPU-side reports)
FP32_FLOP_PER_CLK_PER_SM = 256   # 128 FP32 lanes x FMA
MUFU_OPS_PER_CLK_PER_SM = 16


def device_sm_count(device: int = 0) -> int:
    """Streaming multiprocessors of the CUDA device (cudaDevAttrMultiProcessorCount), or
    GB300_SMS when no device is visible."""
    try:
        import torch

        if torch.cuda.is_available():
            return int(torch.cuda.get_device_properties(device).multi_processor_count)
    except Exception:  # noqa: BLE001 -- a report must not fail on a missing device
        pass
    return GB300_SMS


def ref_rule_evals_per_pair(gauss_qr: int) -> int:
    """Evaluations per triangle pair with the reference rule (9 face-edge entries)."""
    return 9 * gauss_qr * gauss_qr * (gauss_qr - 1) * (gauss_qr - 1)


def measured_peaks(repo_root: str) -> dict:
    path = os.path.join(repo_root, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        d["source"] = "measured"
        return d
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "sm_max_mhz": 2070.0, "source": "fallback"}


def fp32_peak_tflops(sm_mhz: float, sms: int | None = None) -> float:
    sms = device_sm_count() if sms is None else sms
    return sms * FP32_FLOP_PER_CLK_PER_SM * sm_mhz * 1e6 / 1e12


def mufu_peak_gops(sm_mhz: float, sms: int | None = None) -> float:
    sms = device_sm_count() if sms is None else sms
    return sms * MUFU_OPS_PER_CLK_PER_SM * sm_mhz * 1e6 / 1e9
