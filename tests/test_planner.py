"""The statistics planner: its statistics and its plans against the
reference's own (core/gstore.hpp generate_statistic + core/planner.hpp
generate_plan, compiled in place); plans execute to the same rows as the
unplanned query.  Host-only contexts: no GPU needed."""
import numpy as np
import pytest

import oracle
import wukonggpu_gb300 as W
from wukonggpu_gb300 import workloads


@pytest.fixture(scope="module")
def host_ctx(small_graph):
    g, s, p, o = small_graph
    rc = W.RCache(device=-1)
    rc.build_store(s, p, o, g.num_ids)
    return rc


@pytest.fixture(scope="module")
def ref_store(small_graph):
    if not oracle.ref_available():
        pytest.skip("reference sources not present on this machine")
    g, s, p, o = small_graph
    return oracle.RefStore(s, p, o, g.num_ids, keys_million=16, memstore_mb=1024)


def test_host_only_context_refuses_device_work(host_ctx):
    with pytest.raises(W.WkError) as e:
        host_ctx.execute([W.VID_BASE, 2, W.OUT, -1])
    assert e.value.status == W.WK_EDEVICE


def test_statistics_match_reference(host_ctx, ref_store, small_graph):
    g, s, p, o = small_graph
    for which in (0, 1, 2, 3):
        for pid in range(1, g.num_ids + 1):
            assert host_ctx.stat(which, pid) == ref_store.stat(which, pid), (which, pid)
    for a in range(1, g.num_ids + 1):
        for b in range(a + 1, g.num_ids + 1):
            assert host_ctx.stat(4, a, b) == ref_store.stat(4, a, b), (a, b)


def test_plans_match_reference(host_ctx, ref_store, small_graph):
    g, s, p, o = small_graph
    qs = workloads.random_bgps(s, p, o, 300, seed=5, first_class=g.first_class, n_classes=10)
    for q in qs:
        mine, _ = host_ctx.plan(q)
        ref = ref_store.plan(q)
        assert mine == ref, (q, mine, ref)


from wukonggpu_gb300.plans import match_plan as _match  # noqa: E402


def test_plans_give_the_same_rows(host_ctx, small_graph, small_oracle):
    """A plan reorders patterns and renames variables; the bindings are the same.
    Compared through variable names: the planner renumbers in order of first
    appearance, so the planned column of each original variable is recovered
    by matching patterns."""
    g, s, p, o = small_graph
    qs = workloads.random_bgps(s, p, o, 80, seed=9, max_pat=4, first_class=g.first_class, n_classes=10)
    checked = 0
    for q in qs:
        plan, cost = host_ctx.plan(q)
        if not plan:
            continue
        vmap = _match(q, plan)
        assert vmap is not None, (q, plan)
        got, _ = small_oracle.execute(plan)
        # reference: the query as written, constant pattern first, through the oracle
        base = [q[i:i + 4] for i in range(0, len(q), 4)]
        ti = next((i for i, t in enumerate(base) if t[1] == W.TYPE_ID and 0 < t[3] < W.VID_BASE), None)
        if ti is not None:                    # ?x rdf:type C  ->  start from the type index of C
            a, pp, dd, b = base.pop(ti)
            base.insert(0, [b, W.TYPE_ID, W.IN, a])
        else:
            ci = next(i for i, t in enumerate(base) if t[0] >= W.VID_BASE or t[3] >= W.VID_BASE)
            base.insert(0, base.pop(ci))
            if base[0][0] < W.VID_BASE:      # constant at the end: traverse it backwards
                a, pp, dd, b = base[0]
                base[0] = [b, pp, W.IN, a]
        flat = [x for t in base for x in t]
        try:
            exp, _ = small_oracle.execute(flat)
        except ValueError:
            continue                          # the written order is not executable left to right
        # express both in original variable order
        nv = max(-x for x in q if x < 0)
        planned_cols = [-vmap[-(k + 1)] - 1 for k in range(nv)]
        conv = {}
        for t in base:
            for x in (t[0], t[3]):
                if x < 0:
                    conv.setdefault(x, len(conv))
        base_cols = [conv[-(k + 1)] for k in range(nv)]
        a = oracle.canonical(got[:, planned_cols]) if got.size else np.zeros((0, nv), np.int32)
        b = oracle.canonical(exp[:, base_cols]) if exp.size else np.zeros((0, nv), np.int32)
        assert np.array_equal(a, b), (q, plan)
        checked += 1
    assert checked >= 10


def test_plans_match_reference_fixture(host_ctx, golden_small):
    """The reference planner's plans, recorded by tests/golden/gen_golden.py."""
    for rec in golden_small["plans"]:
        mine, _ = host_ctx.plan(rec["bgp"])
        assert mine == rec["plan"], rec


def test_executable_queries_are_left_as_written(host_ctx):
    """The planner's input is SPARQL triple form.  A query already in the
    engine's executable form (IN steps, an index start) gets no plan and is run
    as written, never re-read as triples."""
    for q in ([W.VID_BASE + 5, 2, W.IN, -1],
              [17, W.TYPE_ID, W.IN, -1, -1, 2, W.OUT, -2],
              [2, W.PREDICATE_ID, W.OUT, -1, -1, 2, W.IN, -2]):
        pq, cost = host_ctx.plan(q)
        assert pq == [] and cost == float("inf"), q


def test_planned_heavy_shapes_keep_their_bindings(host_ctx, small_graph, small_oracle):
    """The serving mix's heavy shapes, written as triples, planned by the
    statistics planner, bind the same rows as their executable form."""
    from wukonggpu_gb300 import plans, workloads
    g, s, p, o = small_graph
    layout = workloads.Layout(8, 0, 7, 10, 200_000)   # ids only: 2..9 and 10..16 as the two predicate groups
    assert layout.first_class == g.first_class
    layout.m2o = layout.m2o + [2]                      # the shapes take 8 of each group
    for q, ex in zip(workloads.serving_heavy_queries(layout), workloads.executable_heavy_queries(layout)):
        pq, _ = host_ctx.plan(q)
        assert pq, q
        cols = plans.plan_columns(q, pq)
        a, _ = small_oracle.execute(pq)
        b, _ = small_oracle.execute(ex)
        A = oracle.canonical(a[:, cols]) if a.size else a.reshape(0, len(cols))
        assert A.shape == b.shape and np.array_equal(A, oracle.canonical(b)), (q, pq)
