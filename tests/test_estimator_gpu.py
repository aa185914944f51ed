"""The learned estimator: GPU gradients against the numpy oracle, training,
and the trained model against the statistics estimate on engine-recorded
cardinalities; learned plans give the same bindings as statistics plans."""
import numpy as np
import pytest

import oracle
import wukonggpu_gb300 as W
from oracle import mlp_ref
from wukonggpu_gb300 import estimator, workloads

pytestmark = pytest.mark.gpu


def _rand_batch(rng, M, n_ids):
    feats = rng.normal(0, 1, size=(M, 48)).astype(np.float32)
    pids = rng.integers(0, n_ids + 1, size=M).astype(np.int32)
    tgt = rng.normal(2, 1, size=M).astype(np.float32)
    return feats, pids, tgt


@pytest.mark.parametrize("M", [1, 77, 300])
def test_gradients_match_cpu_oracle(gpu_small, M):
    n_ids = 26
    est = W.Estimator(gpu_small, n_ids, max_batch=512, seed=5)
    rng = np.random.default_rng(M)
    params = est.get_params()
    params += rng.normal(0, 0.01, size=params.shape).astype(np.float32)   # non-zero biases too
    est.set_params(params)
    feats, pids, tgt = _rand_batch(rng, M, n_ids)
    g_gpu, loss_gpu = est.gradients(feats, pids, tgt)
    loss_ref, g_ref = mlp_ref.forward_backward(params, n_ids, feats, pids, tgt)
    # tolerance: BF16 products with FP32 accumulation against the same BF16 roundings
    assert abs(loss_gpu - loss_ref) <= 1e-2 * max(1.0, abs(loss_ref))
    W1 = 256 * 80
    blocks = {"W1": (0, W1), "W2": (W1, W1 + 65536), "W3": (W1 + 65536, W1 + 131072),
              "W4": (W1 + 131072, W1 + 131328), "biases": (W1 + 131328, W1 + 131328 + 832),
              "emb": (W1 + 131328 + 832, len(g_ref))}
    for name, (a, b) in blocks.items():
        x, y = g_gpu[a:b].astype(np.float64), g_ref[a:b].astype(np.float64)
        ny = np.linalg.norm(y)
        if ny == 0:
            assert np.linalg.norm(x) <= 1e-6, name
            continue
        cos = float(x @ y / (np.linalg.norm(x) * ny + 1e-30))
        rel = float(np.linalg.norm(x - y) / ny)
        print(f"gradient block {name} M={M}: cos {cos:.6f} rel {rel:.5f}")
        # the largest relative error seen on a GB300 is 0.00052 (the same BF16
        # roundings; FP32 sums in a different order): a tenfold margin
        assert cos > 0.99999 and rel < 0.005, (name, cos, rel)


def test_training_fits_a_function(gpu_small):
    est = W.Estimator(gpu_small, 26, max_batch=1024, seed=3)
    rng = np.random.default_rng(0)
    feats, pids, _ = _rand_batch(rng, 4000, 26)
    tgt = (feats[:, :4].sum(1) * 0.7 + 0.3 * pids + np.sin(feats[:, 5])).astype(np.float32)
    first = est.train(feats, pids, tgt, epochs=1, batch=256, lr=1e-3)
    last = est.train(feats, pids, tgt, epochs=30, batch=256, lr=1e-3)
    assert last < 0.1 * first, (first, last)


def test_learned_beats_statistics_and_plans_keep_bindings(gpu_small, small_graph, small_oracle):
    g, s, p, o = small_graph
    bgps = workloads.random_bgps(s, p, o, 1500, seed=31, first_class=g.first_class, n_classes=10)
    ds = estimator.build_dataset(gpu_small, bgps)
    tr, te = estimator.split(ds, 0.9, seed=1)
    est = W.Estimator(gpu_small, g.num_ids, max_batch=2048, seed=7)
    est.train(tr["feats"], tr["pids"], tr["target"], epochs=40, batch=512, lr=2e-3)
    ev = estimator.evaluate(est, te)
    assert ev["samples"] > 100
    assert ev["learned_median"] <= ev["stats_median"], ev
    assert ev["learned_p95"] <= ev["stats_p95"], ev
    # learned plans execute to the same bindings as the statistics plans
    from wukonggpu_gb300.plans import match_plan as _match
    checked = 0
    for q in bgps[:150]:
        sp, _ = gpu_small.plan(q)
        lp, _ = est.plan(q)
        if not sp or not lp:
            continue
        ms, ml = _match(q, sp), _match(q, lp)
        assert ms is not None and ml is not None, (q, sp, lp)
        a, _ = small_oracle.execute(sp)
        b, _ = small_oracle.execute(lp)
        nv = max(-x for x in q if x < 0)
        ca = [-ms[-(k + 1)] - 1 for k in range(nv)]
        cb = [-ml[-(k + 1)] - 1 for k in range(nv)]
        A = oracle.canonical(a[:, ca]) if a.size else np.zeros((0, nv), np.int32)
        B = oracle.canonical(b[:, cb]) if b.size else np.zeros((0, nv), np.int32)
        assert np.array_equal(A, B), (q, sp, lp)
        checked += 1
    assert checked >= 50


def test_batched_learned_planning_equals_single(gpu_small, small_graph):
    g, s, p, o = small_graph
    bgps = workloads.random_bgps(s, p, o, 200, seed=41, first_class=g.first_class, n_classes=10)
    est = W.Estimator(gpu_small, g.num_ids, max_batch=4096, seed=9)
    many = est.plan_many(bgps)
    for q, pm in zip(bgps, many):
        single, _ = est.plan(q)
        assert pm == single


def test_row_limit_is_an_error_not_a_truncation(gpu_small, golden_small):
    q = next(x for x in golden_small["queries"] if x["name"] == "pindex_out")
    gpu_small.set_row_limit(1000)
    try:
        with pytest.raises(W.WkError) as e:
            gpu_small.execute(q["cmd_chains"])
        assert e.value.status == W.WK_EOVERFLOW
    finally:
        gpu_small.set_row_limit(0)
    req, _ = gpu_small.execute(q["cmd_chains"])
    assert req.result_table.shape[0] == q["rows"]


def test_untrusted_model_falls_back_to_statistics_plans(gpu_small, small_graph):
    """A model whose held-out q-error exceeds the stated bound is not used: the
    learned planners return exactly the statistics planner's plans."""
    g, s, p, o = small_graph
    bgps = workloads.random_bgps(s, p, o, 300, seed=53, first_class=g.first_class, n_classes=10)
    ds = estimator.build_dataset(gpu_small, bgps[:150])
    est = W.Estimator(gpu_small, g.num_ids, max_batch=4096, seed=13)   # untrained
    assert est.trusted
    p95, ok = est.validate(ds["feats"], ds["pids"], ds["target"], qerror_bound=2.0)
    assert not ok and p95 > 2.0 and not est.trusted
    many = est.plan_many(bgps)
    n_stats = 0
    for q, pm in zip(bgps, many):
        sp, _ = gpu_small.plan(q)
        single, _ = est.plan(q)
        assert single == pm
        if sp:
            assert single == sp
            n_stats += 1
    assert n_stats > 200
    # a bound the model meets restores it
    p95b, okb = est.validate(ds["feats"], ds["pids"], ds["target"], qerror_bound=p95 * 2 + 1.0)
    assert okb and est.trusted


def test_learned_planner_leaves_executable_queries_as_written(gpu_small, small_graph):
    """Like the statistics planner, the learned one plans SPARQL triple form
    only: an IN step or an index start means the query is already executable."""
    g, s, p, o = small_graph
    est = W.Estimator(gpu_small, g.num_ids, max_batch=1024, seed=3)
    qs = [[W.VID_BASE + 5, 2, W.IN, -1],
          [g.first_class, W.TYPE_ID, W.IN, -1, -1, 2, W.OUT, -2],
          [2, W.PREDICATE_ID, W.OUT, -1, -1, 2, W.IN, -2]]
    for q in qs:
        assert est.plan(q)[0] == [], q
    assert est.plan_many(qs) == [[], [], []]
