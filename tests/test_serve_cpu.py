"""Host-side serving logic that needs no GPU: HBM budget admission."""
import threading
import time

import pytest

from rocket_gb300.serve import Budget


def test_budget_blocks_until_release():
    b = Budget(100.0)
    b.reserve(60.0)
    got = []

    def second():
        b.reserve(50.0)
        got.append(time.perf_counter())

    t = threading.Thread(target=second)
    t0 = time.perf_counter()
    t.start()
    time.sleep(0.2)
    assert not got  # 60 + 50 > 100: waits
    b.release(60.0)
    t.join(5)
    assert got and got[0] - t0 >= 0.2
    assert b.used == 50.0 and b.peak == 60.0


def test_budget_refuses_what_can_never_fit():
    b = Budget(10.0)
    with pytest.raises(MemoryError):
        b.reserve(11.0)


def test_budget_times_out():
    b = Budget(10.0)
    b.reserve(8.0)
    with pytest.raises(TimeoutError):
        b.reserve(5.0, timeout=0.1)
