"""Batched execution: every query's table equals the one it produces alone
(same rows, same order) -- against the oracle and against the single-query
GPU path -- through graph replays of different batches, tuning changes and
capacity limits."""
import numpy as np
import pytest

import oracle
import wukonggpu_gb300 as W
from wukonggpu_gb300 import workloads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def light(small_graph):
    g, s, p, o = small_graph
    return workloads.light_queries(s, p, o, 600, seed=3)


def _check(tables, queries, orc):
    for t, q in zip(tables, queries):
        exp, _ = orc.execute(q)
        got = t.reshape(exp.shape) if t.size == 0 else t
        assert got.shape == exp.shape and np.array_equal(got, exp), q


@pytest.mark.parametrize("threads", [256, 128])
@pytest.mark.parametrize("fused", [False, True])
def test_batch_matches_oracle_graph_and_plain(gpu_small, small_oracle, light, fused, threads):
    """Both step forms (three kernels per step, or one cooperative kernel
    whose blocks meet at grid barriers) at both block sizes."""
    b = W.Batch(gpu_small, max_queries=1024, max_steps=4, capacity_ints=1 << 24)
    b.set_fused(fused)
    assert b.fused() == fused
    b.set_block_threads(threads)
    assert b.block_threads() == threads
    for use_graph in (False, True):
        k0 = b.kernel_launches()
        nq = b.run(light, use_graph=use_graph)
        _check(b.download(nq), light, small_oracle)
        assert b.kernel_launches() - k0 == 1 + (1 if fused else 3) * 4
    for bps, rows, split in ((2, 32, 16), (8, 128, 256)):   # 8 blocks/SM: clamped to what fits at once
        b.set_tuning(bps, rows, split)
        nq = b.run(light[:300])
        _check(b.download(nq), light[:300], small_oracle)


@pytest.mark.parametrize("threads", [256, 128])
def test_fused_batch_of_one_query(gpu_small, small_oracle, light, threads):
    """The one-kernel step on the smallest batch: one query, whose rows fill a
    fraction of one tile while every block of the grid meets at the barriers."""
    b = W.Batch(gpu_small, max_queries=1, max_steps=4, capacity_ints=1 << 22)
    b.set_fused(True)
    b.set_block_threads(threads)
    for i in (0, 7, 100):
        b.run([light[i]])
        _check(b.download(1), [light[i]], small_oracle)


def test_fused_batch_capacity_overflow_is_reported(gpu_small, light):
    """The scan inside the one-kernel step finds the overflow; every block
    leaves after the barrier and later steps do nothing."""
    b = W.Batch(gpu_small, max_queries=1024, max_steps=4, capacity_ints=4096)
    b.set_fused(True)
    with pytest.raises(W.WkError) as e:
        b.run(light)
    assert e.value.status == W.WK_EOVERFLOW


def test_graph_replay_with_new_batches(gpu_small, small_oracle, small_graph):
    g, s, p, o = small_graph
    b = W.Batch(gpu_small, max_queries=1024, max_steps=4, capacity_ints=1 << 24)
    for seed in (11, 12, 13):
        qs = workloads.light_queries(s, p, o, 512, seed=seed)
        nq = b.run(qs)
        _check(b.download(nq), qs, small_oracle)


def test_alone_equals_in_the_mix(gpu_small, light):
    b = W.Batch(gpu_small, max_queries=1024, max_steps=4, capacity_ints=1 << 24)
    nq = b.run(light)
    mixed = [t.copy() for t in b.download(nq)]
    for i in (0, 7, 100, 599):
        b1 = W.Batch(gpu_small, max_queries=1, max_steps=4, capacity_ints=1 << 22)
        b1.run([light[i]])
        alone = b1.download(1)[0]
        assert np.array_equal(alone, mixed[i])
        req, _ = gpu_small.execute(light[i])              # the single-query path
        assert np.array_equal(req.result_table.reshape(alone.shape) if alone.size == 0 else req.result_table, alone)


def test_tuning_and_autotune_keep_results(gpu_small, small_oracle, light):
    b = W.Batch(gpu_small, max_queries=1024, max_steps=4, capacity_ints=1 << 24)
    for bps, rows, split in ((2, 32, 16), (8, 128, 256), (4, 64, 1)):
        b.set_tuning(bps, rows, split)
        nq = b.run(light[:300])
        _check(b.download(nq), light[:300], small_oracle)
    ms = b.autotune(light, reps=2)
    assert ms > 0 and b.tuning()[0] in (2, 4, 8)
    three, one = b.autotune_forms()        # each step form's best; the kept one is the faster
    assert three is not None and one is not None
    assert min(three, one) == pytest.approx(ms)
    assert b.fused() == (one < three)
    assert b.block_threads() in (128, 256)
    nq = b.run(light)
    _check(b.download(nq), light, small_oracle)


def test_capacity_overflow_is_reported(gpu_small, light):
    b = W.Batch(gpu_small, max_queries=1024, max_steps=4, capacity_ints=4096)
    b.set_block_threads(128)               # the tile sums are sized for the smaller tiles
    with pytest.raises(W.WkError) as e:
        b.run(light)
    assert e.value.status == W.WK_EOVERFLOW


def test_bad_batch_queries_rejected(gpu_small):
    b = W.Batch(gpu_small, max_queries=8, max_steps=2, capacity_ints=1 << 16)
    with pytest.raises(W.WkError):
        b.run([[W.VID_BASE, 2, W.OUT, -1, -1, 2, W.OUT, -2, -2, 2, W.OUT, -3]])   # 3 patterns > 2
    with pytest.raises(W.WkError):
        b.run([[-1, 2, W.OUT, -2]])                                               # no constant start


def test_index_starts_in_a_batch(gpu_small, small_oracle, small_graph, light):
    """Type-index and predicate-index starts run in a batch (as the list of the
    index key) beside constant starts, each with the rows it has alone."""
    g, s, p, o = small_graph
    C0 = g.first_class
    qs = [[C0, W.TYPE_ID, W.IN, -1, -1, 2, W.OUT, -2],
          [C0 + 1, W.TYPE_ID, W.IN, -1, -1, 3, W.OUT, -2, -2, 5, W.OUT, -3],
          [4, W.PREDICATE_ID, W.OUT, -1, -1, 4, W.IN, -2],
          [6, W.PREDICATE_ID, W.IN, -1, -1, 6, W.OUT, -2, -1, W.TYPE_ID, W.OUT, -3]] + light[:60]
    b = W.Batch(gpu_small, max_queries=128, max_steps=4, capacity_ints=1 << 24)
    tabs = b.download(b.run(qs))
    for q, t in zip(qs, tabs):
        exp, _ = small_oracle.execute(q)
        assert np.array_equal(oracle.canonical(t), oracle.canonical(exp)), q
    with pytest.raises(W.WkError):
        b.run([[C0, W.TYPE_ID, W.OUT, -1]])      # a type index is an IN list
