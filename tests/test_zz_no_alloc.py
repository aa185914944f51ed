"""The allocation-free known_to_unknown against the ordinary one.

Callers that cannot allocate device memory mid-query (a host running the
operator inside its own allocator callback or under a fixed device budget, a
serving thread that must never enter cudaMalloc) use
wk_known_to_unknown_noalloc with buffers they already own.  This file is
collected last so that a failure here cannot hide other tests; it passes both
alone in a fresh process and after the rest of the suite.
"""
import ctypes as C

import numpy as np
import pytest

import wukonggpu_gb300 as W

pytestmark = pytest.mark.gpu

MAX_ROWS = 1 << 18


def _noalloc(rc, hist_ptr, rows, cols, start, d, pid, out_ptr, cap):
    lib = W.load_library()
    nrows = C.c_int64(-1)
    st = lib.wk_known_to_unknown_noalloc(rc._h, hist_ptr, rows, cols, start, d, pid, out_ptr, cap,
                                         C.byref(nrows))
    return st, nrows.value


def _download(owner, ptr, rows, cols):
    h = W.wk_history()
    h.data = ptr
    h.size = rows * cols
    h.col_num = cols
    out = np.zeros(max(h.size, 1), np.int32)
    assert W.load_library().wk_history_download(owner._h, C.byref(h), out.ctypes.data_as(W._I32P), out.size) == 0
    return out[:h.size].reshape(-1, cols)


@pytest.fixture(scope="module")
def setup():
    g = W.Graph(W.spec_small())
    s, p, o = (np.array(a) for a in g.arrays())
    rc = W.RCache(device=0)
    rc.build_store_graph(g)
    out_owner = W.RCache(device=0)         # owns the caller's output buffer
    return g, s, rc, out_owner


def _history(s, R, C, seed):
    rng = np.random.default_rng(seed)
    h = rng.choice(np.unique(s), size=(R, C)).astype(np.int32)
    h[rng.random((R, C)) < 0.25] = W.VID_BASE + 50_000_000
    return h


def _free_device_bytes():
    torch = pytest.importorskip("torch")
    return torch.cuda.mem_get_info(0)[0]


# (input rows, columns, predicate, direction): output widths 3, 4, 8 (the
# widest specialised expansion) and 10 (the generic one with scalar stores);
# the maximum row count; a small call whose output ends inside a 16 B group
@pytest.mark.parametrize("R,C,pid,d", [(70_001, 3, 2, W.OUT), (MAX_ROWS, 2, 5, W.IN), (4_099, 7, 3, W.OUT),
                                       (3_001, 9, 4, W.IN), (5, 2, 2, W.OUT)])
def test_noalloc_matches_existing_op_twice(setup, R, C, pid, d):
    g, s, rc, out_owner = setup
    cap = 16 << 20
    outreq = W.Request([])
    out_owner.upload_history(outreq, np.zeros((cap, 1), np.int32))
    out_ptr = outreq.hist.data
    for call, seed in enumerate((R, R + 1)):           # two calls in a row, different inputs
        h = _history(s, R, C, seed)
        req = W.Request([])
        rc.upload_history(req, h)
        in_ptr = req.hist.data
        rc.sync()
        free0 = _free_device_bytes()
        st, nrows = _noalloc(rc, in_ptr, R, C, -1 - (call % C), d, pid, out_ptr, cap)
        assert st == W.WK_OK, W.load_library().wk_last_error()
        # the call took no device memory (no allocation, no module load)
        assert _free_device_bytes() == free0
        got = _download(out_owner, out_ptr, nrows, C + 1)
        rc.known_to_unknown(req, -1 - (call % C), d, pid)      # the ordinary entry point
        exp = rc.download(req)
        assert exp.shape == got.shape and np.array_equal(got, exp), call


def test_noalloc_rejects_oversize_and_small_output(setup):
    g, s, rc, out_owner = setup
    req = W.Request([])
    rc.upload_history(req, _history(s, 1000, 2, 3))
    st, _ = _noalloc(rc, req.hist.data, MAX_ROWS + 1, 2, -1, W.OUT, 2, None, 0)
    assert st == W.WK_EINVAL and b"maximum" in W.load_library().wk_last_error()
    small = W.Request([])
    out_owner.upload_history(small, np.zeros((8, 1), np.int32))
    st, nrows = _noalloc(rc, req.hist.data, 1000, 2, -1, W.OUT, 2, small.hist.data, 8)
    assert st == W.WK_EOVERFLOW and nrows > 2


def test_noalloc_rejects_unaligned_buffers(setup):
    """Output rows are written as 16 B vectors: an output pointer off a 16 B
    boundary (and a history pointer off a 4 B boundary) is refused on the host,
    before any kernel runs."""
    g, s, rc, out_owner = setup
    req = W.Request([])
    rc.upload_history(req, _history(s, 100, 2, 5))
    dst = W.Request([])
    out_owner.upload_history(dst, np.zeros((4096, 1), np.int32))
    base = C.cast(dst.hist.data, C.c_void_p).value
    hbase = C.cast(req.hist.data, C.c_void_p).value
    st, _ = _noalloc(rc, req.hist.data, 100, 2, -1, W.OUT, 2, C.cast(C.c_void_p(base + 4), W._I32P), 4000)
    assert st == W.WK_EINVAL and b"aligned" in W.load_library().wk_last_error()
    st, _ = _noalloc(rc, C.cast(C.c_void_p(hbase + 2), W._I32P), 99, 2, -1, W.OUT, 2, dst.hist.data, 4096)
    assert st == W.WK_EINVAL and b"aligned" in W.load_library().wk_last_error()
