"""The Izhikevich update's binary64 arithmetic on the integer pipe, and its float-float evaluation,
equal the hardware FP64 pipe's results."""
import pytest

from braingrid_gb300 import lib as bg

pytestmark = pytest.mark.gpu


def test_integer_binary64_matches_hardware():
    add, mul, conv, outside = bg.selftest_binary64(samples=1 << 27, seed=12345)
    assert (add, mul, conv) == (0, 0, 0), (add, mul, conv)
    assert outside < (1 << 27) // 1000  # exponent sums leaving the normal range are rare here


def test_izhikevich_expression_three_ways():
    """The whole double expression of the Izhikevich update on 2^26 random operand sets: the
    integer-pipe restatement and the float-float evaluation give the FP64 pipe's floats; the
    float-float evaluation hands only a small fraction of values back to the FP64 pipe."""
    n = 1 << 26
    soft, ff, handed, outside = bg.selftest_izhikevich(samples=n, seed=777)
    assert soft == 0 and ff == 0, (soft, ff)
    assert handed < n // 200, handed
    assert outside < n // 1000, outside
