"""Device-side safety paths, exercised without a fault: a bounded copy wait on a
barrier that nothing completes gives up after its limit and reports it (the
solver's copy stages then end the solve with an error instead of spinning)."""
import pytest

from am_ml_suite_gb300 import _native as nat


@pytest.mark.gpu
@pytest.mark.parametrize("limit_ms", [2.0, 10.0])
def test_bounded_copy_wait_gives_up(limit_ms):
    timed_out, waited = nat.selftest_copy_wait(limit_ms)
    assert timed_out
    assert limit_ms <= waited < limit_ms + 50.0


def test_copy_wait_limits_are_checked():
    with pytest.raises(nat.AmError):
        nat.selftest_copy_wait(0.0)
    with pytest.raises(nat.AmError):
        nat.selftest_copy_wait(1000.0)
