"""vkhel_measure_int_peak: the integer-pipe denominators of the transform
rooflines, checked against what the hardware can issue.

A GB300 SM issues 64 32-bit IMADs per clock (the heavy half of the FMA pipe),
so the measured IMAD rate must lie at or below 64 x SMs x the maximum SM
clock (a few percent of timing slack) and, on an idle GPU running at or near
that clock, not far below it.  A lazy Cooley-Tukey butterfly costs about 22
IMAD-class issue slots (one 64x64 high product and two low products, plus
the integer adds), so the butterfly rate sits between 1/40 and 1/12 of the
IMAD rate.
"""
import subprocess

import pytest

pytestmark = pytest.mark.gpu


def _max_sm_mhz():
    try:
        out = subprocess.run(["nvidia-smi", "-i", "0", "--query-gpu=clocks.max.sm", "--format=csv,noheader,nounits"],
                             capture_output=True, text=True, timeout=30).stdout
        return float(out.split()[0])
    except (OSError, ValueError, IndexError, subprocess.SubprocessError):
        pytest.skip("nvidia-smi clocks unavailable")


def test_int_peak_matches_the_issue_rate(vk, ctx):
    bfly, imad = ctx.measure_int_peak()
    sms = ctx.sm_count
    ceiling = 64.0 * sms * _max_sm_mhz() * 1e6
    assert imad <= 1.03 * ceiling, (imad, ceiling)
    assert imad >= 0.6 * ceiling, (imad, ceiling)
    assert imad / 40 <= bfly <= imad / 12, (bfly, imad)
