"""Host-side logic of bench.py (no GPU): the host-link bound of the e2e
roofline and the link warm-up."""
import os
import sys

import pytest

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
import bench  # noqa: E402

RATES = {"h2d": 211.4, "d2h": 193.4, "duplex": [172.0, 171.6]}


def test_host_link_bound_of_the_ct_mult_step():
    # 1024 pairs at n = 2^14, six limbs: 3.2 GB in, 1.6 GB out.
    ct = 2 * 6 * (1 << 14) * 8
    ms = bench.host_link_ms(2 * 1024 * ct, 1024 * ct, RATES)
    # copy-out beside copy-in for 9.39 ms, then 1.61 GB alone at 211.4 GB/s
    assert ms == pytest.approx(16.98, abs=0.02)


def test_host_link_bound_limits():
    # nothing back: the copy-in alone at the one-way rate
    assert bench.host_link_ms(211.4e6, 0, RATES) == pytest.approx(1.0)
    # nothing in: the copy-out alone at the one-way rate
    assert bench.host_link_ms(0, 193.4e6, RATES) == pytest.approx(1.0)
    # more out than in: 1 ms side by side, then the rest of the copy-out alone
    assert bench.host_link_ms(172.0e6, 171.6e6 + 193.4e6, RATES) == pytest.approx(2.0)
    # the bound never beats either direction alone
    for bi, bo in ((3e9, 1e9), (1e9, 3e9), (2e9, 2e9)):
        ms = bench.host_link_ms(bi, bo, RATES)
        assert ms >= bi / (RATES["h2d"] * 1e6) - 1e-9
        assert ms >= bo / (RATES["d2h"] * 1e6) - 1e-9


def test_warm_link_runs_at_least_the_calls_and_the_time():
    calls = []
    bench.warm_link(lambda: calls.append("step"), lambda: calls.append("sync"), 3, seconds=0)
    assert calls == ["step", "sync"] * 3
    calls.clear()
    bench.warm_link(lambda: calls.append("step"), lambda: None, 1, seconds=0.05)
    assert len(calls) > 1
