"""The measured roofline denominator: the integer ALU-pipe rate of the device."""
import pytest

import bwacuda as B

pytestmark = pytest.mark.gpu


def test_alu_peak_is_plausible(ctx):
    g = ctx.measure_alu_peak()
    # 152 SMs x 64 lanes x ~2 GHz is about 2e4 Gop/s; allow for clocks and other SM counts
    assert 2000.0 < g < 60000.0, g


def test_op_rates(ctx):
    # every DPX form the kernels use issues as one ALU-pipe instruction: its rate is the ALU peak's
    peak = ctx.measure_alu_peak()
    rates = ctx.measure_op_rates()
    assert set(rates) == set(B.OP_RATE_NAMES)
    assert all(v > 0 for v in rates.values())
    for name in ("viaddmax_s32", "viaddmax_s16x2", "viaddmax_s16x2_relu", "vimax3_s16x2", "vimax3_u16x2"):
        assert 0.8 * peak < rates[name] < 1.25 * peak, (name, rates[name], peak)


def test_host_link(ctx):
    # the link the host-buffer calls use: every rate positive and below a generous physical bound
    r = ctx.measure_host_link(64 << 20)
    assert set(r) == {"device_read_gbs", "copy_h2d_gbs", "device_write_gbs"}
    assert all(0 < v < 2000 for v in r.values()), r
    with pytest.raises(B.BwaCudaError):
        ctx.measure_host_link(1000)  # below 1 MiB
