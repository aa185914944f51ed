"""Weighted template mixes in the reference batch driver's format
(scripts/batch/mix_config, core/proxy.hpp:287-457) and the reference Logger's
per-type statistics (core/logger.hpp:182-305)."""
import numpy as np
import pytest

import oracle
import wukonggpu_gb300 as W
from wukonggpu_gb300 import mix as M
from wukonggpu_gb300 import workloads

MIX = M.MIX_DIR / "serving" / "mix_config"


def test_get_distribution_follows_the_reference_rule():
    """utils/mymath.hpp:28-41: r modulo the weights' sum, then the first type
    whose cumulative weight exceeds it."""
    w = [3, 1, 6]
    assert [M.get_distribution(r, w) for r in range(10)] == [0, 0, 0, 1, 2, 2, 2, 2, 2, 2]
    assert M.get_distribution(10, w) == 0 and M.get_distribution(13, w) == 1
    with pytest.raises(ValueError):
        M.get_distribution(1, [0, 0])


def test_parse_packaged_mix():
    types = M.parse_mix(MIX)
    assert len(types) == 10 and sum(t.heavy for t in types) == 4
    assert [t.heavy for t in types] == [False] * 6 + [True] * 4     # heavy types come last
    light = sum(t.weight for t in types if not t.heavy)
    assert light / sum(t.weight for t in types) == pytest.approx(0.95)
    assert all(t.placeholders for t in types if not t.heavy)
    assert not any(t.placeholders for t in types if t.heavy)


def test_parse_rejects_malformed(tmp_path):
    (tmp_path / "a.tpl").write_text("%C0 F1 OUT -1\n")
    (tmp_path / "h.q").write_text("%C0 TYPE IN -1\n")
    (tmp_path / "m1").write_text("2 1\na.tpl 5\n")
    with pytest.raises(ValueError):
        M.parse_mix(tmp_path / "m1")                    # header counts two types
    (tmp_path / "m2").write_text("2 1\na.tpl 5\nh.q 1\n")
    with pytest.raises(ValueError):
        M.parse_mix(tmp_path / "m2")                    # a heavy query with a random constant
    (tmp_path / "m3").write_text("1 0\na.tpl 0\n")
    with pytest.raises(ValueError):
        M.parse_mix(tmp_path / "m3")                    # weights are positive


@pytest.fixture(scope="module")
def serving_small(lib_built):
    """The serving generator at 1/200 of its entities (about 5M triples)."""
    g = W.Graph(W.spec_serving(scale=0.005))
    s, p, o = (np.array(a) for a in g.arrays())
    layout = workloads.Layout(16, 32, 16, 15, int(g.spec.n_entities))
    return g, s, p, o, layout


def test_instantiate_and_draw(serving_small):
    """Every random constant of a request comes from one seed: member
    seed % n of its class (core/query.hpp:198-205); types follow the weights."""
    g, s, p, o, layout = serving_small
    rc = W.RCache(device=-1)
    rc.build_store(s, p, o, g.num_ids)
    mx = M.Mix(MIX, layout)
    mx.fill_candidates(rc)
    members = rc.get_edges(0, layout.first_class + 1, W.IN)
    q = mx.instantiate(mx.types[1], 12345)                 # light_q2: %C1 M1 OUT -1 / -1 M1 IN -2
    assert q == [int(members[12345 % len(members)]), layout.m2o[0], W.OUT, -1, -1, layout.m2o[0], W.IN, -2]
    # the class of a drawn constant is its template's class
    t = dict(zip((int(x) for x in s[p == W.TYPE_ID]), (int(x) for x in o[p == W.TYPE_ID])))
    reqs = mx.draw(4000, seed=3)
    for k, q in reqs[:200]:
        for (i, j, c) in mx.types[k].placeholders:
            assert t[q[4 * i + j]] == layout.first_class + c
    counts = np.bincount([k for k, _ in reqs], minlength=len(mx.types)) / len(reqs)
    expect = np.array(mx.weights) / sum(mx.weights)
    assert np.all(np.abs(counts - expect) < 0.03)
    heavy = [q for k, q in reqs if mx.types[k].heavy]
    tf = M.Mix.triple_form(heavy[0])
    assert tf[:4] == [-1, W.TYPE_ID, W.OUT, heavy[0][0]] and tf[4:] == heavy[0][4:]


@pytest.mark.gpu
def test_typed_serving_statistics_and_results(serving_small):
    """A weighted mix through the request loop: every request's rows equal the
    oracle's, and each type's p50/p99 and 25-point CDF are the Logger's
    statistics of that type's own latencies."""
    from oracle import logger_ref
    g, s, p, o, layout = serving_small
    rc = W.RCache(device=0)
    rc.build_store_graph(g)
    mx = M.Mix(MIX, layout)
    mx.fill_candidates(rc)
    reqs = mx.draw(2500, seed=9)
    srv = W.Server(rc, mode=1, plan=0, max_batch=1024, heavy_workers=2, batch_capacity_ints=1 << 26)
    arr = W.poisson_arrivals(len(reqs), rate_qps=40_000.0, seed=4)
    ids = [srv.submit(q, float(t), qtype=k) for (k, q), t in zip(reqs, arr)]
    srv.start()
    srv.drain(300)
    orc = oracle.Oracle(s, p, o, g.num_ids)
    lat = {k: [] for k in range(len(mx.types))}
    for rid, (k, q) in zip(ids, reqs):
        got, l, status = srv.result(rid)
        exp, _ = orc.execute(q)
        assert status == 0
        if mx.types[k].heavy:       # index start: the reference's index order is not fixed
            assert oracle.rows_digest(got) == oracle.rows_digest(exp), mx.types[k].name
        else:
            assert np.array_equal(got.reshape(exp.shape) if got.size == 0 else got, exp), mx.types[k].name
        lat[k].append(l * 1e3)
    for k, t in enumerate(mx.types):
        ts = srv.type_stats(k)
        assert ts["completed"] == len(lat[k]) > 0 and ts["failed"] == 0, t.name
        assert ts["p50_ms"] == pytest.approx(logger_ref.at_rate(lat[k], 0.50), rel=1e-9)
        assert ts["p99_ms"] == pytest.approx(logger_ref.at_rate(lat[k], 0.99), rel=1e-9)
        assert ts["cdf_ms"] == pytest.approx(logger_ref.cdf(lat[k]), rel=1e-9)
    assert srv.type_stats(99)["completed"] == 0
    srv.close()
    rc.close()
