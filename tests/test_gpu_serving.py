"""Serving loop: requests admitted by HBM budget run concurrently on the
device, and each result equals the request run alone."""
import numpy as np
import pytest

from q1tsim_gb300.serving import Request, Server, latency_stats, mixed_requests, run_alone, serve

pytestmark = pytest.mark.gpu


def test_results_same_alone_and_in_the_mix():
    reqs = mixed_requests(24, seed=3, qmin=8, qmax=15, dmin=3, dmax=12, shots=512)
    done, wall, srv = serve(reqs, rate_hz=20000, hbm_budget_bytes=1 << 30, slots=4)
    assert len(done) == len(reqs)
    assert all(r.error is None for r in done), [r.error for r in done if r.error]
    assert srv.peak_inflight > 1, "requests should overlap on the device"
    for r in reqs:
        assert np.array_equal(run_alone(r), r.result), r.rid
    stats = latency_stats(done)
    assert stats["completed"] == len(reqs) and stats["p99_ms"] >= stats["p50_ms"]


def test_admission_respects_the_hbm_budget():
    reqs = mixed_requests(12, seed=8, qmin=12, qmax=16, dmin=2, dmax=6, shots=256)
    budget = max(r.state_bytes() for r in reqs) * 2
    done, wall, srv = serve(reqs, rate_hz=50000, hbm_budget_bytes=budget, slots=6)
    assert len(done) == 12 and all(r.error is None for r in done)
    assert srv.peak_used <= budget
    big = Request(99, reqs[0].circuit, 256, 1)
    small = Server(hbm_budget_bytes=16, slots=1)
    with pytest.raises(ValueError):
        small.submit(big)
    small.close()
