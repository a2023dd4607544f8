"""The Izhikevich update's binary64 arithmetic on the integer pipe equals the hardware's."""
import pytest

from braingrid_gb300 import lib as bg

pytestmark = pytest.mark.gpu


def test_integer_binary64_matches_hardware():
    add, mul, conv, outside = bg.selftest_binary64(samples=1 << 27, seed=12345)
    assert (add, mul, conv) == (0, 0, 0), (add, mul, conv)
    assert outside < (1 << 27) // 1000  # exponent sums leaving the normal range are rare here
