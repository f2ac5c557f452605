"""The algorithmic bytes behind every roofline fraction (eff_pot_gb300/roofline.py).

Each fused stage of a steppc step reads its inputs once and writes its outputs
once; per step at N points (FP64): predictor 168 N, corrector 152 N, two
poten evaluations of 108 N (OT), plus about 272 N each for the alpha_s and
gradient terms of OTC: 536 N for OT, about 1080 N for OTC, half in FP32.  The
per-kernel model of roofline.py must add up to those totals.
"""
import pytest

from eff_pot_gb300.roofline import step_bytes


@pytest.mark.parametrize("n", [64, 128, 192])
def test_step_bytes_match_the_stage_count(n):
    N = n ** 3
    for s in (8, 4):
        ot = sum(step_bytes(n, n, n, otc=False, grad=False, s=s, renorm=False).values())
        otc = sum(step_bytes(n, n, n, otc=True, grad=True, s=s, renorm=False).values())
        assert abs(ot / N - 536 * s / 8) < 0.03 * 536 * s / 8
        assert abs(otc / N - 1080 * s / 8) < 0.03 * 1080 * s / 8


def test_fp32_is_half_of_fp64():
    b8 = step_bytes(128, 128, 128, s=8, renorm=False)
    b4 = step_bytes(128, 128, 128, s=4, renorm=False)
    assert b8.keys() == b4.keys()
    for k in b8:
        assert b8[k] == 2 * b4[k], k
