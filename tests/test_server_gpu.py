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


@pytest.mark.parametrize("mode", [0, 1])
def test_latency_statistics_follow_the_logger(gpu_small, mix, mode):
    """p50/p99 and the 25-point CDF, overall and per class, are the reference
    Logger's statistics (core/logger.hpp:197-305) of the requests' own
    latencies.  The class (light: a constant start of at most max_steps
    patterns; heavy: an index start) is the request's shape in both modes, so
    the query-at-a-time baseline reports both classes too."""
    from oracle import logger_ref
    srv = W.Server(gpu_small, mode=mode, plan=0, max_batch=1024)
    arr = W.poisson_arrivals(len(mix), rate_qps=30_000.0 if mode else 8_000.0, seed=3)
    ids = [srv.submit(q, float(t)) for q, t in zip(mix, arr)]
    srv.start()
    srv.drain(300)
    lats = [srv.result(i, fetch=False)[1] * 1e3 for i in ids]
    light = [x for x, q in zip(lats, mix) if q[0] >= W.VID_BASE]
    heavy = [x for x, q in zip(lats, mix) if q[0] < W.VID_BASE]
    assert light and heavy
    st = srv.stats()
    assert st["light"] == len(light) and st["heavy"] == len(heavy)
    assert st["p50_ms"] == pytest.approx(logger_ref.at_rate(lats, 0.50), rel=1e-9)
    assert st["p99_ms"] == pytest.approx(logger_ref.at_rate(lats, 0.99), rel=1e-9)
    assert st["light_p99_ms"] == pytest.approx(logger_ref.at_rate(light, 0.99), rel=1e-9)
    assert st["heavy_p99_ms"] == pytest.approx(logger_ref.at_rate(heavy, 0.99), rel=1e-9)
    assert st["light_p99_ms"] > 0 and st["heavy_p99_ms"] > 0
    cdf = srv.latency_cdf("all")
    assert cdf == pytest.approx(logger_ref.cdf(lats), rel=1e-9)
    assert srv.latency_cdf("light") == pytest.approx(logger_ref.cdf(light), rel=1e-9)
    assert srv.latency_cdf("heavy") == pytest.approx(logger_ref.cdf(heavy), rel=1e-9)
    assert W.Server.CDF_RATES == pytest.approx(logger_ref.cdf_rates())
    srv.close()


def _check_results(srv, ids, mix, orc, skip=()):
    for rid, q in zip(ids, mix):
        if rid in skip:
            continue
        got, _, status = srv.result(rid)
        exp, _ = orc.execute(q)
        assert status == 0
        assert np.array_equal(got.reshape(exp.shape) if got.size == 0 else got, exp), q


def test_cancel_and_admission_refusal_leave_other_results_unchanged(gpu_small, small_oracle, mix):
    """Requests cancelled before they start and requests refused at admission
    (projected history bytes over the cap) complete with their own status and
    no rows; every other request of the mix gives the rows it gives alone."""
    srv = W.Server(gpu_small, mode=1, plan=0, max_batch=512, heavy_workers=2, batch_capacity_ints=1 << 24,
                   max_request_bytes=4 << 20)
    arr = W.poisson_arrivals(len(mix), rate_qps=50_000.0, seed=11)
    ids = [srv.submit(q, float(t)) for q, t in zip(mix, arr)]
    refused = {rid for rid in ids if srv.finished(rid) and srv.result(rid, fetch=False)[2] == W.WK_EREJECTED}
    assert refused, "the cap refuses no request of the mix"
    cancel = [rid for rid in ids[::37] if rid not in refused]
    for rid in cancel:
        assert srv.cancel(rid)
    assert not srv.cancel(cancel[0])                 # already cancelled: finished
    srv.start()
    srv.drain(300)
    st = srv.stats()
    assert st["rejected"] == len(refused) and st["cancelled"] == len(cancel)
    assert st["completed"] == len(mix) - len(refused) - len(cancel) and st["failed"] == 0
    for rid in cancel:
        got, _, status = srv.result(rid)
        assert status == W.WK_ECANCELED and got.size == 0
    for rid in refused:
        assert srv.result(rid, fetch=False)[2] == W.WK_EREJECTED
    _check_results(srv, ids, mix, small_oracle, skip=set(cancel) | refused)
    srv.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_injected_allocation_failure_fails_only_its_requests(gpu_small, small_oracle, mix, mode):
    """A worker whose next device-buffer reservations fail (injected on the
    host, as a failed cudaMalloc would) fails exactly that many requests with
    WK_ENOMEM; the server keeps serving and every other result is unchanged."""
    srv = W.Server(gpu_small, mode=mode, plan=0, max_batch=512, heavy_workers=1, batch_capacity_ints=1 << 24)
    arr = W.poisson_arrivals(len(mix), rate_qps=20_000.0, seed=12)
    ids = [srv.submit(q, float(t)) for q, t in zip(mix, arr)]
    srv.inject_alloc_failure(0, 3)
    srv.start()
    srv.drain(300)
    st = srv.stats()
    failed = [rid for rid in ids if srv.result(rid, fetch=False)[2] != 0]
    assert len(failed) == 3 and st["failed"] == 3
    assert all(srv.result(rid, fetch=False)[2] == W.WK_ENOMEM for rid in failed)
    _check_results(srv, ids, mix, small_oracle, skip=set(failed))
    srv.close()


def test_injected_allocation_failure_on_a_context(gpu_small, small_oracle, golden_small):
    """An op that meets an injected allocation failure returns WK_ENOMEM and
    changes nothing: the next query on the same context is exact."""
    q = golden_small["queries"][0]["cmd_chains"]
    gpu_small.inject_alloc_failure(1)
    with pytest.raises(W.WkError) as e:
        gpu_small.execute(q)
    assert e.value.status == W.WK_ENOMEM
    req, rows = gpu_small.execute(q)
    exp, erows = small_oracle.execute(q)
    assert list(rows) == list(erows)
    assert np.array_equal(W.canonical_rows(req.result_table), W.canonical_rows(exp))
