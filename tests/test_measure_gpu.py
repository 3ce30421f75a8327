"""The measured roofline denominator: the integer ALU-pipe rate of the device."""
import pytest

pytestmark = pytest.mark.gpu


def test_alu_peak_is_plausible(ctx):
    g = ctx.measure_alu_peak()
    # 152 SMs x 64 lanes x ~2 GHz is about 2e4 Gop/s; allow for clocks and other SM counts
    assert 2000.0 < g < 60000.0, g
