"""Parity of the CUDA path with the oracle and the reference fixtures.

Every comparison is bit-exact.  Non-index queries must match the reference
row order exactly; index-start queries match in canonical order (the
reference fills its index lists from racing loader threads) and match the
oracle exactly (both keep index lists ascending)."""
import hashlib

import numpy as np
import pytest

import oracle
import wukonggpu_gb300 as W
from wukonggpu_gb300 import workloads

pytestmark = pytest.mark.gpu


def _sha(t):
    return hashlib.sha256(np.ascontiguousarray(t, np.int32).tobytes()).hexdigest()


def test_store_matches_oracle_keys(gpu_small, small_oracle):
    info = gpu_small.store_info()
    assert info["num_keys"] == small_oracle.num_keys()
    d, k, e = small_oracle.digest()
    assert info["num_edges"] == e
    assert info["overflow_buckets"] > 0          # chains are exercised


def test_host_lookup_matches_oracle(gpu_small, small_graph, small_oracle):
    g, s, p, o = small_graph
    rng = np.random.default_rng(3)
    verts = rng.choice(np.unique(np.concatenate([s, o[p != 1]])), 300, replace=False)
    for v in verts:
        for pid in (1, 2, 5, 9):
            for d in (W.IN, W.OUT):
                assert np.array_equal(gpu_small.get_edges(int(v), pid, d), small_oracle.get_edges(int(v), pid, d))


def test_golden_queries(gpu_small, small_oracle, golden_small):
    for q in golden_small["queries"]:
        req, rows = gpu_small.execute(q["cmd_chains"])
        t = req.result_table
        assert t.shape[0] == q["rows"], q["name"]
        assert list(rows) == q["step_rows"], q["name"]
        assert _sha(oracle.canonical(t)) == q["canonical_sha256"], q["name"]
        if "ordered_sha256" in q:
            assert _sha(t) == q["ordered_sha256"], q["name"]
        ref, _ = small_oracle.execute(q["cmd_chains"])
        assert np.array_equal(t.reshape(ref.shape) if t.size else ref, ref), q["name"]


def _random_history(rng, verts, R, C, miss_frac=0.3):
    h = rng.choice(verts, size=(R, C)).astype(np.int32)
    miss = rng.random((R, C)) < miss_frac
    h[miss] = W.VID_BASE + 10_000_000 + rng.integers(0, 1000, size=miss.sum())
    return h


@pytest.mark.parametrize("R", [1, 31, 33, 1023, 1025, 4097, 70_001])
@pytest.mark.parametrize("C", [1, 2, 3, 4, 5, 6, 7, 8])   # every specialised output width, and one above
def test_k2u_random_histories(gpu_small, small_graph, small_oracle, R, C):
    g, s, p, o = small_graph
    rng = np.random.default_rng(R * 7 + C)
    verts = np.unique(s)
    h = _random_history(rng, verts, R, C)
    for pid, d in ((2, W.OUT), (3, W.IN), (1, W.OUT)):
        scol = int(rng.integers(0, C))
        req = W.Request([])
        gpu_small.upload_history(req, h)
        gpu_small.known_to_unknown(req, -scol - 1, d, pid)
        got = gpu_small.download(req)
        exp, _ = small_oracle.step(h, False, -scol - 1, pid, d, -C - 1)
        assert got.shape == exp.shape and np.array_equal(got, exp), (pid, d, scol)


def test_interleaved_op_sizes_on_a_fresh_context(small_graph, small_oracle):
    """One new context, ops of growing and shrinking size: each op's totals
    reach the host through pinned memory, whose buffer grows when an op has
    more groups than any before it (1, 3, 1, 3 and 11 groups here, k2u and
    k2k ops alternating)."""
    g, s, p, o = small_graph
    rc = W.RCache(device=0)
    rc.build_store_graph(g)
    rng = np.random.default_rng(77)
    verts = np.unique(s)
    m = p == 2
    es, eo = s[m], o[m]
    try:
        for R, kind in ((1000, "k2u"), (700_001, "k2u"), (3000, "k2u"), (700_001, "k2k"), (2_800_003, "k2u"),
                        (5, "k2k"), (2_800_003, "k2k"), (1, "k2u")):
            C = 3
            h = _random_history(rng, verts, R, C, miss_frac=0.1)
            if kind == "k2k":   # rows that are real edges, so that some are kept
                idx = rng.integers(0, len(es), size=R)
                real = rng.random(R) < 0.5
                h[real, 0] = es[idx[real]]
                h[real, 1] = eo[idx[real]]
            req = W.Request([])
            rc.upload_history(req, h)
            if kind == "k2u":
                rc.known_to_unknown(req, -2, W.OUT, 2)
                exp, _ = small_oracle.step(h, False, -2, 2, W.OUT, -C - 1)
            else:
                rc.known_to_known(req, -1, W.OUT, 2, -2)
                exp, _ = small_oracle.step(h, False, -1, 2, W.OUT, -2)
            st = rc.last_op_stats()
            got = rc.download(req)
            assert np.array_equal(got.reshape(exp.shape), exp), (R, kind)
            # the op's two kernels and the publish kernel; a k2u op with no
            # output rows launches no expansion
            assert st["kernels"] == (3 if kind == "k2k" or len(exp) else 2), (R, kind)
    finally:
        rc.close()


@pytest.mark.parametrize("R", [1, 33, 1025, 50_000, 700_001])   # 700,001 rows: 684 blocks in 3 groups of 256
@pytest.mark.parametrize("C", [2, 5, 11])
def test_k2k_k2c_random_histories(gpu_small, small_graph, small_oracle, R, C):
    g, s, p, o = small_graph
    rng = np.random.default_rng(R + 13 * C)
    # rows that are real edges (so matches occur) mixed with random pairs
    m = p == 2
    es, eo = s[m], o[m]
    idx = rng.integers(0, len(es), size=R)
    h = _random_history(rng, np.unique(s), R, C, miss_frac=0.1)
    real = rng.random(R) < 0.6
    h[real, 0] = es[idx[real]]
    h[real, 1] = eo[idx[real]]
    for (start, d, pid, end) in ((-1, W.OUT, 2, -2), (-2, W.IN, 2, -1), (-1, W.OUT, 3, -2)):
        req = W.Request([])
        gpu_small.upload_history(req, h)
        gpu_small.known_to_known(req, start, d, pid, end)
        got = gpu_small.download(req)
        exp, _ = small_oracle.step(h, False, start, pid, d, end)
        assert np.array_equal(got.reshape(exp.shape), exp), (start, d, pid, end)
    vals, counts = np.unique(eo, return_counts=True)
    for const in (int(vals[np.argmax(counts)]), int(vals[0]), W.VID_BASE + 99_999_999):
        req = W.Request([])
        gpu_small.upload_history(req, h)
        gpu_small.known_to_const(req, -1, W.OUT, 2, const)
        got = gpu_small.download(req)
        exp, _ = small_oracle.step(h, False, -1, 2, W.OUT, const)
        assert np.array_equal(got.reshape(exp.shape), exp), const


# 2,599,000 rows: 2,539 blocks in 10 groups, the last block ragged
@pytest.mark.parametrize("R", [1, 33, 4097, 60_000, 600_000, 2_599_000])
def test_k2k_k2c_on_a_functional_direction(gpu_small, small_graph, small_oracle, R):
    """rdf:type OUT is dense and functional: its membership test reads the
    neighbour array once.  Rows mix real (entity, class) pairs, wrong classes,
    absent vertices and index keys (0, looked up in the hash table)."""
    g, s, p, o = small_graph
    rng = np.random.default_rng(R)
    m = p == W.TYPE_ID
    es, eo = s[m], o[m]
    idx = rng.integers(0, len(es), size=R)
    h = np.stack([es[idx], eo[idx], es[rng.integers(0, len(es), size=R)]], 1).astype(np.int32)
    wrong = rng.random(R) < 0.4
    h[wrong, 1] = 17 + rng.integers(0, 10, size=wrong.sum())
    h[rng.random(R) < 0.05, 0] = W.VID_BASE + 50_000_000
    h[rng.random(R) < 0.02, 0] = 0
    for (start, end) in ((-1, -2), (-3, -2)):
        req = W.Request([])
        gpu_small.upload_history(req, h)
        gpu_small.known_to_known(req, start, W.OUT, W.TYPE_ID, end)
        got = gpu_small.download(req)
        exp, _ = small_oracle.step(h, False, start, W.TYPE_ID, W.OUT, end)
        assert np.array_equal(got.reshape(exp.shape), exp), (start, end)
    for const in (17, 21, 5):
        req = W.Request([])
        gpu_small.upload_history(req, h)
        gpu_small.known_to_const(req, -1, W.OUT, W.TYPE_ID, const)
        got = gpu_small.download(req)
        exp, _ = small_oracle.step(h, False, -1, W.TYPE_ID, W.OUT, const)
        assert np.array_equal(got.reshape(exp.shape), exp), const


def test_index_and_const_starts(gpu_small, small_graph, small_oracle):
    g, s, p, o = small_graph
    for idx, d in ((17, W.IN), (20, W.IN), (2, W.IN), (2, W.OUT), (16, W.OUT)):
        req = W.Request([])
        gpu_small.index_to_unknown(req, idx, d)
        got = gpu_small.download(req).reshape(-1)
        exp, _ = small_oracle.step(None, True, idx, 0, d, -1)
        assert np.array_equal(got, exp.reshape(-1)), (idx, d)
    for v in np.unique(s)[:50]:
        req = W.Request([])
        gpu_small.const_to_unknown(req, int(v), W.OUT, 2)
        got = gpu_small.download(req).reshape(-1)
        assert np.array_equal(got, small_oracle.get_edges(int(v), 2, W.OUT))


def test_empty_history_steps(gpu_small):
    req = W.Request([])
    gpu_small.upload_history(req, np.zeros((0, 3), np.int32))
    gpu_small.known_to_unknown(req, -2, W.OUT, 2)
    assert req.hist.size == 0 and req.hist.col_num == 4
    gpu_small.known_to_known(req, -1, W.OUT, 2, -4)
    assert req.hist.size == 0 and req.hist.col_num == 4


def test_bad_patterns_are_errors(gpu_small):
    req = W.Request([])
    gpu_small.upload_history(req, np.full((4, 2), W.VID_BASE, np.int32))
    with pytest.raises(W.WkError) as e:
        gpu_small.known_to_unknown(req, -3, W.OUT, 2)     # column 2 is not bound
    assert e.value.status == W.WK_EINVAL
    with pytest.raises(W.WkError):
        gpu_small.known_to_unknown(req, -1, W.OUT, 999)   # predicate out of range
    with pytest.raises(W.WkError):
        gpu_small.known_to_unknown(req, -1, 2, 2)         # direction
    with pytest.raises(W.WkError):
        gpu_small.execute([W.VID_BASE + 1, 2, W.OUT, -1, -1, 2, W.OUT, -3])   # skips a column
    with pytest.raises(W.WkError):
        gpu_small.execute([-1, 2, W.OUT, -2])               # starts from an unknown variable


def _hub_graph():
    """A graph with one subject of degree 5000 (k2u rows spanning many write
    tiles), a functional chain for wide tables, and ordinary random edges."""
    rng = np.random.default_rng(11)
    n = 20_000
    V = W.VID_BASE
    hub = V
    s = [np.full(3000, hub), V + rng.integers(0, n, 40_000), V + np.arange(n)]
    o = [V + 1 + np.arange(3000), V + rng.integers(0, n, 40_000), V + (np.arange(n) * 7919 + 1) % n]
    pp = [np.full(3000, 2), np.full(40_000, 2), np.full(n, 3)]
    s = np.concatenate(s).astype(np.int32)
    o = np.concatenate(o).astype(np.int32)
    pp = np.concatenate(pp).astype(np.int32)
    # type triples
    s = np.concatenate([s, V + np.arange(n)]).astype(np.int32)
    o = np.concatenate([o, 4 + (np.arange(n) % 3)]).astype(np.int32)
    pp = np.concatenate([pp, np.ones(n, np.int32)]).astype(np.int32)
    return s, pp, o, 6


def test_high_degree_and_wide_tables(lib_built):
    s, p, o, nid = _hub_graph()
    rc = W.RCache(device=0)
    rc.build_store(s, p, o, nid)
    orc = oracle.Oracle(s, p, o, nid)
    hubq = [W.VID_BASE, 2, W.OUT, -1, -1, 2, W.IN, -2, -2, 2, W.OUT, -3]
    req, rows = rc.execute(hubq)
    exp, erows = orc.execute(hubq)
    assert list(rows) == list(erows) and np.array_equal(req.result_table, exp)
    # 26-column table through a functional chain (the reference stops at 20 columns)
    q = [4, W.TYPE_ID, W.IN, -1]
    for i in range(25):
        q += [-(i + 1), 3, W.OUT, -(i + 2)]
    req, rows = rc.execute(q)
    exp, erows = orc.execute(q)
    assert req.result_table.shape == exp.shape == (exp.shape[0], 26)
    assert np.array_equal(req.result_table, exp)


def test_paged_segment_cache_gives_same_rows(small_graph, small_oracle, golden_small):
    g, s, p, o = small_graph
    # the store is ~26 MB, its largest segment (the type lists) ~2.5 MB: the
    # queries' segments do not fit together, a step's pair does
    rc = W.RCache(device=0, cache_budget_mb=5)
    rc.build_store_graph(g)
    assert rc.store_info()["paged"] == 1
    for q in golden_small["queries"]:
        req, rows = rc.execute(q["cmd_chains"])
        assert _sha(oracle.canonical(req.result_table)) == q["canonical_sha256"], q["name"]
        assert list(rows) == q["step_rows"], q["name"]
    info = rc.store_info()
    assert info["cache_loads"] > 0 and info["cache_evictions"] > 0


def test_fragmented_segment_cache_compacts(small_graph, small_oracle):
    """A pool whose free bytes would hold a segment but whose free ranges do
    not (the current step's segment, kept resident, splits them) is compacted
    instead of refusing the segment (the reference pages fixed frames,
    core/shard_manager.hpp:78-128; here a segment is one range, moved down).

    Budget 5 MiB; segments 2, 3 and 6 (about 1.6 MB each) are loaded in that
    order, then a query steps through 3 and then the type segment (2.4 MB),
    with 3 still protected (the prefetch finds no free space and leaves the
    load to the step): evicting 2 and 6 frees 3.6 MB in two ranges of at most
    2.0 MB around 3."""
    g, s, p, o = small_graph
    host = W.RCache(device=-1)
    host.build_store(s, p, o, g.num_ids)
    size = {pid: host.seg_layout(pid)["device_bytes"] for pid in (1, 2, 3, 6)}
    budget = 5 << 20
    assert size[2] + size[3] + size[6] <= budget < size[2] + size[3] + size[6] + size[1]
    assert max(size[2], size[6] + budget - size[2] - size[3] - size[6]) < size[1] <= budget - size[3]
    rc = W.RCache(device=0, cache_budget_mb=5, enable_prefetch=True)
    rc.build_store_graph(g)
    for pid in (2, 3, 6):                       # one-pattern queries: no prefetch, one segment each
        c = int(s[p == pid][0])
        req, _ = rc.execute([c, pid, W.OUT, -1])
        assert np.array_equal(req.result_table.reshape(-1), small_oracle.get_edges(c, pid, W.OUT))
    c = int(s[p == 3][0])
    q = [c, 3, W.OUT, -1, -1, W.TYPE_ID, W.OUT, -2]
    req, rows = rc.execute(q)
    exp, erows = small_oracle.execute(q)
    assert list(rows) == list(erows) and np.array_equal(req.result_table, exp)
    info = rc.store_info()
    assert info["cache_compactions"] >= 1 and info["cache_evictions"] >= 2
    assert info["cache_hits"] < info["cache_requests"]
    # every segment still answers after the move
    for pid in (3, 1):
        req, _ = rc.execute([c, pid, W.OUT, -1])
        assert np.array_equal(req.result_table.reshape(-1), small_oracle.get_edges(c, pid, W.OUT))


def test_kernel_launch_count_and_timing(gpu_small, golden_small):
    before = gpu_small.kernel_launches()
    gpu_small.enable_timing(True)
    q = next(x for x in golden_small["queries"] if x["name"] == "type_chain")
    gpu_small.execute(q["cmd_chains"])
    st = gpu_small.last_op_stats()
    gpu_small.enable_timing(False)
    assert gpu_small.kernel_launches() > before
    assert st["kernels"] == 3 and st["ms"] > 0 and st["ms_main"] > 0   # k2u: count + publish + expand
    assert st["rows_out"] == q["rows"]


def test_functional_direction_reaching_an_index_list(lib_built):
    """A functional direction expands as a compaction; a history value 0 looks
    up the index key [0|p|d] (core/gstore.hpp:389-409), a long list, and the op
    must still give the reference's rows."""
    s, p, o, nid = _hub_graph()
    rc = W.RCache(device=0)
    rc.build_store(s, p, o, nid)
    orc = oracle.Oracle(s, p, o, nid)
    assert rc.store_info()["dense_dirs"] > 0
    rng = np.random.default_rng(5)
    h = (W.VID_BASE + rng.integers(0, 20_000, size=(3000, 2))).astype(np.int32)
    for with_zero in (False, True):
        if with_zero:
            h[1500, 0] = 0
        for d in (W.OUT, W.IN):
            req = W.Request([])
            rc.upload_history(req, h)
            rc.known_to_unknown(req, -1, d, 3)
            got = rc.download(req)
            exp, _ = orc.step(h, False, -1, 3, d, -3)
            assert got.shape == exp.shape and np.array_equal(got, exp), (with_zero, d)


def test_sparse_functional_direction(lib_built):
    """A functional predicate whose subjects are sparse in the id range: its OUT
    direction stays hashed (with a presence bitmap) and still takes the one-pass
    functional k2u; rows, order and misses equal the oracle's."""
    rng = np.random.default_rng(17)
    V = W.VID_BASE
    n = 50_000
    subj = V + np.arange(0, n, 40)                            # 1 in 40 ids: hashed, not dense
    s = np.concatenate([subj, V + rng.integers(0, n, 30_000), V + np.arange(n)]).astype(np.int32)
    o = np.concatenate([V + rng.integers(0, n, len(subj)), V + rng.integers(0, n, 30_000),
                        np.full(n, 3)]).astype(np.int32)
    p = np.concatenate([np.full(len(subj), 2), np.full(30_000, 4), np.ones(n)]).astype(np.int32)
    rc = W.RCache(device=0)
    rc.build_store(s, p, o, 4)
    orc = oracle.Oracle(s, p, o, 4)
    for C in (1, 3, 7):
        h = (V + rng.integers(0, n, size=(20_011, C))).astype(np.int32)
        h[::7, 0] = subj[rng.integers(0, len(subj), size=len(h[::7]))]   # many hits among misses
        req = W.Request([])
        rc.upload_history(req, h)
        rc.known_to_unknown(req, -1, W.OUT, 2)
        got = rc.download(req)
        exp, _ = orc.step(h, False, -1, 2, W.OUT, -C - 1)
        assert got.shape == exp.shape and np.array_equal(got, exp), C


def test_query_op_stats_cover_every_pattern(gpu_small, golden_small):
    q = next(x for x in golden_small["queries"] if x["name"] == "type_chain")
    gpu_small.enable_timing(True)
    req, rows = gpu_small.execute(q["cmd_chains"])
    stats = gpu_small.query_op_stats()
    gpu_small.enable_timing(False)
    assert len(stats) == len(q["cmd_chains"]) // 4
    assert [s["rows_out"] for s in stats] == list(rows)
    assert all(s["ms"] > 0 for s in stats if s["rows_out"] > 0)
    assert stats[0]["kind"] == 3 and all(s["kind"] in (0, 1, 2) for s in stats[1:])


@pytest.mark.parametrize("which", ["small", "hub", "dups", "classpred"])
def test_device_sorted_build_gives_the_same_image(lib_built, small_graph, which):
    """wk_store_build_device builds the image on the GPU (sorts, lists,
    dense arrays, bitmaps, bucket insertion); the image (buckets, edges,
    offsets arrays, metadata) must be byte-identical to the host build's."""
    if which == "small":
        g, s, p, o = small_graph
        nid = g.num_ids
    else:
        s, p, o, nid = _hub_graph()
        if which == "dups":   # duplicates and a shuffled order
            rng = np.random.default_rng(8)
            k = rng.integers(0, len(s), size=len(s) // 3)
            s, p, o = (np.concatenate([x, x[k]]) for x in (s, p, o))
            perm = rng.permutation(len(s))
            s, p, o = s[perm], p[perm], o[perm]
        if which == "classpred":   # id 5 is a class and a predicate: two [0|5|IN] index keys
            rng = np.random.default_rng(9)
            m = 5000
            s = np.concatenate([s, W.VID_BASE + rng.integers(0, 20_000, m)]).astype(np.int32)
            p = np.concatenate([p, np.full(m, 5)]).astype(np.int32)
            o = np.concatenate([o, W.VID_BASE + rng.integers(0, 20_000, m)]).astype(np.int32)
    a = W.RCache(device=0)
    a.build_store(s, p, o, nid)
    b = W.RCache(device=0)
    b.build_store(s, p, o, nid, on_device=True)
    assert a.store_digest() == b.store_digest()
    assert a.store_info()["num_keys"] == b.store_info()["num_keys"]


@pytest.mark.parametrize("bad", ["predicate", "subject", "class", "object"])
def test_device_build_refuses_bad_triples_as_the_host_does(lib_built, bad):
    s, p, o, nid = _hub_graph()
    s, p, o = s.copy(), p.copy(), o.copy()
    i = int(np.flatnonzero(p == W.TYPE_ID)[7]) if bad == "class" else 1234
    if bad == "predicate":
        p[i] = nid + 1
    elif bad == "subject":
        s[i] = 5
    elif bad == "class":
        o[i] = nid + 3
    else:
        o[i] = -7
    p[i + 5] = 0   # a later bad triple: the first one is reported
    msgs = []
    for dev in (False, True):
        rc = W.RCache(device=0)
        with pytest.raises(W.WkError) as e:
            rc.build_store(s, p, o, nid, on_device=dev)
        assert e.value.status == W.WK_EINVAL
        msgs.append(str(e.value))
        rc.close()
    assert msgs[0] == msgs[1]


def test_k2u_over_256_groups(lib_built):
    """An op of more than 256 x 256 input blocks (67.1M rows): each expansion
    CTA finds its block from the per-group sums in more than one pass.  The
    general (fan-out) and the functional expansion are checked row for row
    against a vectorised expansion of the oracle's adjacency lists."""
    V = W.VID_BASE
    n = 1000
    v = np.arange(n)
    fan = np.where(v % 4 == 0, 3, np.where(v % 4 == 1, 1, 0))   # 1 neighbour per vertex on average
    s2 = np.repeat(v, fan)
    j = np.arange(len(s2)) - np.repeat(np.cumsum(fan) - fan, fan)
    o2 = (s2 * 7 + j * 13) % n
    s3 = v[v % 2 == 0]
    o3 = (s3 * 31 + 7) % n
    s = np.concatenate([s2, s3, v]) + V
    o = np.concatenate([o2 + V, o3 + V, np.full(n, 4)])
    p = np.concatenate([np.full(len(s2), 2), np.full(len(s3), 3), np.ones(n)])
    s, p, o = s.astype(np.int32), p.astype(np.int32), o.astype(np.int32)
    rc = W.RCache(device=0)
    rc.build_store(s, p, o, 4)
    orc = oracle.Oracle(s, p, o, 4)
    R = 256 * 256 * 1024 + 391_000
    h = (V + np.random.default_rng(23).integers(0, n, size=(R, 1))).astype(np.int32)
    vals = h[:, 0] - V
    for pid in (2, 3):
        lists = [orc.get_edges(int(x) + V, pid, W.OUT) for x in range(n)]
        deg = np.array([len(x) for x in lists], np.int64)
        offs = np.concatenate([[0], np.cumsum(deg)])
        flat = np.concatenate(lists).astype(np.int32)
        d = deg[vals]
        rows = np.repeat(np.arange(R), d)
        k = np.arange(len(rows)) - np.repeat(np.cumsum(d) - d, d)
        exp = np.stack([h[rows, 0], flat[offs[vals[rows]] + k]], axis=1)
        del rows, k
        req = W.Request([])
        rc.upload_history(req, h)
        rc.known_to_unknown(req, -1, W.OUT, pid)
        got = rc.download(req)
        assert got.shape == exp.shape and np.array_equal(got, exp), pid


@pytest.mark.parametrize("with_index_key", [False, True])
def test_large_functional_k2u(gpu_small, small_graph, small_oracle, with_index_key):
    """A functional op over a 112 MB history (7,000,001 rows: 27 groups, the
    last one ragged), once as the compaction and once with an index key among
    its rows, which makes the op rerun unspecialised."""
    g, s, p, o = small_graph
    rng = np.random.default_rng(5)
    ents = np.unique(s[p == W.TYPE_ID])
    R, C = 7_000_001, 4
    h = rng.choice(ents, size=(R, C)).astype(np.int32)
    h[rng.random(R) < 0.2, 1] = W.VID_BASE + 90_000_000   # no type: the row is dropped
    if with_index_key:
        h[4_500_017, 1] = 0
    req = W.Request([])
    gpu_small.upload_history(req, h)
    gpu_small.known_to_unknown(req, -2, W.OUT, W.TYPE_ID)
    got = gpu_small.download(req)
    exp, _ = small_oracle.step(h, False, -2, W.TYPE_ID, W.OUT, -C - 1)
    assert got.shape == exp.shape and np.array_equal(got, exp)
