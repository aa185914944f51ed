"""The store layout on a host-only context (no GPU): directions whose vertex
keys are dense in their id range are stored as offsets arrays, the rest
hashed; every lookup, through either form, returns the oracle's adjacency list
(core/gstore.hpp:389-409: an absent key is an empty list)."""
import numpy as np
import pytest

import wukonggpu_gb300 as W


@pytest.fixture(scope="module")
def host_store(small_graph):
    g, s, p, o = small_graph
    rc = W.RCache(device=-1)
    rc.build_store(s, p, o, g.num_ids)
    return rc


def test_both_forms_are_used(host_store, small_oracle):
    info = host_store.store_info()
    assert info["dense_dirs"] > 0                 # e.g. the type list of every entity
    assert info["overflow_buckets"] > 0           # hashed directions still chain
    assert info["num_keys"] == small_oracle.num_keys()


def test_lookups_match_oracle(host_store, small_graph, small_oracle):
    g, s, p, o = small_graph
    rng = np.random.default_rng(11)
    verts = np.unique(np.concatenate([s, o[p != 1]]))
    lo, hi = int(verts.min()), int(verts.max())
    present = rng.choice(verts, 400, replace=False)
    # ids inside the range that have no key, and ids on and beyond its ends
    absent = np.setdiff1d(np.arange(lo, hi + 1, 97), verts)[:100]
    edge_ids = [lo - 1, lo, hi, hi + 1, hi + 1000, W.VID_BASE]
    for v in list(present) + list(absent) + edge_ids:
        for pid in range(1, g.num_ids + 1):
            for d in (W.IN, W.OUT):
                assert np.array_equal(host_store.get_edges(int(v), pid, d), small_oracle.get_edges(int(v), pid, d)), \
                    (int(v), pid, d)


def test_index_keys_stay_hashed(host_store, small_graph, small_oracle):
    g, s, p, o = small_graph
    for pid in range(1, g.num_ids + 1):
        for d in (W.IN, W.OUT):
            assert np.array_equal(host_store.get_edges(0, pid, d), small_oracle.get_edges(0, pid, d)), (pid, d)
