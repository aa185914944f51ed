"""The request loop: results of a mixed open-loop load equal each query's
result alone (the oracle on the same plan), in both modes, with and without
the statistics planner; latency accounting is sane."""
import numpy as np
import pytest

import oracle
import wukonggpu_gb300 as W
from wukonggpu_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mix(small_graph, golden_small):
    g, s, p, o = small_graph
    light = workloads.light_queries(s, p, o, 1500, seed=21)
    heavy = [q["cmd_chains"] for q in golden_small["queries"] if 1 < q["cmd_chains"][0] < W.VID_BASE]
    rng = np.random.default_rng(4)
    qs = light + heavy * 3
    order = rng.permutation(len(qs))
    return [qs[i] for i in order]


@pytest.mark.parametrize("mode,plan,window_us", [(0, 0, 0), (1, 0, 0), (1, 1, 0), (1, 0, 400)])
def test_results_alone_equal_results_in_the_mix(gpu_small, small_oracle, mix, mode, plan, window_us):
    srv = W.Server(gpu_small, mode=mode, plan=plan, max_batch=512, heavy_workers=2, batch_capacity_ints=1 << 24,
                   batch_window_us=window_us)
    arr = W.poisson_arrivals(len(mix), rate_qps=50_000.0, seed=1)
    ids = [srv.submit(q, float(t)) for q, t in zip(mix, arr)]
    srv.start()
    srv.drain(300)
    st = srv.stats()
    assert st["completed"] == len(mix) and st["failed"] == 0
    for rid, q in zip(ids, mix):
        cmd = q
        if plan:
            pq, _ = gpu_small.plan(q)
            if pq is None:          # proved empty by the statistics
                got, _, _ = srv.result(rid)
                assert got.size == 0
                continue
            if pq:
                cmd = pq
        got, lat, status = srv.result(rid)
        exp, _ = small_oracle.execute(cmd)
        assert status == 0 and lat >= 0
        assert np.array_equal(got.reshape(exp.shape) if got.size == 0 else got, exp), (q, cmd)
    if mode == 1:
        assert st["batches"] > 0 and st["light"] > 0 and st["heavy"] > 0
    srv.close()


def test_latency_and_throughput_reported(gpu_small, mix):
    srv = W.Server(gpu_small, mode=1, plan=1, max_batch=1024, keep_results=0)
    arr = W.poisson_arrivals(len(mix), rate_qps=20_000.0, seed=2)
    for q, t in zip(mix, arr):
        srv.submit(q, float(t))
    srv.start()
    srv.drain(300)
    st = srv.stats()
    assert st["qps"] > 0 and 0 < st["p50_ms"] <= st["p99_ms"]
    assert st["span_s"] >= arr[-1] - arr[0] - 1e-3
    srv.close()


def test_latency_statistics_follow_the_logger(gpu_small, mix):
    """p50/p99 and the 25-point CDF are the reference Logger's statistics
    (core/logger.hpp:197-305) of the requests' own latencies."""
    from oracle import logger_ref
    srv = W.Server(gpu_small, mode=1, plan=0, max_batch=1024)
    arr = W.poisson_arrivals(len(mix), rate_qps=30_000.0, seed=3)
    ids = [srv.submit(q, float(t)) for q, t in zip(mix, arr)]
    srv.start()
    srv.drain(300)
    lats = [srv.result(i, fetch=False)[1] * 1e3 for i in ids]
    st = srv.stats()
    assert st["p50_ms"] == pytest.approx(logger_ref.at_rate(lats, 0.50), rel=1e-9)
    assert st["p99_ms"] == pytest.approx(logger_ref.at_rate(lats, 0.99), rel=1e-9)
    cdf = srv.latency_cdf("all")
    assert cdf == pytest.approx(logger_ref.cdf(lats), rel=1e-9)
    for cls in ("light", "heavy"):
        c = srv.latency_cdf(cls)
        assert all(a <= b for a, b in zip(c, c[1:])) and c[-1] <= cdf[-1] + 1e-9
    assert W.Server.CDF_RATES == pytest.approx(logger_ref.cdf_rates())
    srv.close()
