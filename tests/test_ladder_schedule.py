"""Host logic of the mixed-precision solver and of the benchmark's units, on CPU.

* The precision ladder: FP8 + BF16 → BF16 → fused split-BF16x3 → split-BF16x3 with separate
  accumulators. A stage ends when the update norm crosses its threshold or stops falling
  (two iterations above 0.8 × the stage's best). The final stage is at its floor after four.
* The flop units of the benchmark against the figures of the scope table: F_iter at
  no=20, nv=180 and no=40, nv=300; F_(T) at no=30, nv=240.
"""
import os
import sys

import pytest

from pycc_gb300.mixed import MixedResidual

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402


class W:
    device1, stream, vvvv_fp8, switch_threshold = "cpu", None, True, 1e-5


def feed(m, norms):
    for r in norms:
        m.select_mode(r)
    return m.history


def test_thresholds_advance_the_ladder():
    m = MixedResidual(W())
    hist = feed(m, [float("inf"), 5e-2, 5e-4, 2e-4, 5e-6])
    # inf: no norm yet; 5e-4 < 1e-3 ends FP8; 5e-6 < 1e-5 ends BF16
    assert hist == ["fp8", "fp8", "bf16", "bf16", "bf16x3f"]


def test_stall_advances_and_final_stage_floor():
    m = MixedResidual(W())
    feed(m, [1e-2, 5e-4])                      # FP8 -> BF16 on the threshold
    assert m.mode_name() == "bf16"
    feed(m, [1e-4, 9e-5, 9e-5])                # two iterations above 0.8 x best: stall
    assert m.mode_name() == "bf16x3f"
    assert not m.at_floor()
    feed(m, [1e-6, 1e-7, 1e-7, 1e-7])          # the fused stage stalls at its floor
    assert m.mode_name() == "bf16x3s"
    feed(m, [5e-8, 4.5e-8, 4.5e-8, 4.5e-8])
    assert not m.at_floor()                    # three non-improving iterations
    feed(m, [4.5e-8])
    assert m.at_floor()                        # four: the solver takes the last four energies


def test_final_stage_request():
    m = MixedResidual(W())
    m.select_mode(0.0)                         # explicit request for the final stage
    assert m.mode_name() == "bf16x3s" and m.is_final_mode()


def test_single_stage_modes():
    assert MixedResidual(W(), mode="bf16x6").stages == ["bf16x6"]
    assert MixedResidual(W(), mode="bf16x3").stages == ["bf16x3"]

    class W2(W):
        vvvv_fp8 = False
    assert MixedResidual(W2()).stages == ["bf16", "bf16x3f", "bf16x3s"]


def test_flop_units():
    assert bench.f_iter(20, 180) == pytest.approx(1.72e12, rel=5e-3)
    assert bench.f_iter(40, 300) == pytest.approx(5.84e13, rel=5e-3)
    assert 2 * 40**2 * 300**4 == pytest.approx(2.59e13, rel=5e-3)       # the ladder term
    assert 2 * 30**3 * 240**4 + 2 * 30**4 * 240**3 == pytest.approx(2.02e14, rel=5e-3)
