"""The C ABI library: it loads, exports every symbol the header declares, and
reports errors as statuses (no compute call needs a GPU here)."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

import wukonggpu_gb300 as W

HEADER = Path(__file__).resolve().parents[1] / "include" / "wukong_gpu.h"


def _declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(wk_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_op_surface():
    names = _declared()
    for n in ("wk_known_to_unknown", "wk_known_to_known", "wk_known_to_const", "wk_index_to_unknown",
              "wk_const_to_unknown", "wk_execute", "wk_store_build", "wk_ctx_create"):
        assert n in names


def test_library_exports_every_declared_symbol(lib_built):
    lib = C.CDLL(str(W.lib_path()))
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_mirror_covers_header(lib_built):
    assert set(_declared()) <= set(W.exported_symbols())


def test_status_strings(lib_built):
    lib = W.load_library()
    for st in (W.WK_OK, W.WK_EINVAL, W.WK_ENOMEM, W.WK_ETIMEDOUT, W.WK_EDEVICE, W.WK_ENOSTORE, W.WK_EOVERFLOW):
        assert lib.wk_status_str(st)


def test_null_arguments_are_rejected(lib_built):
    lib = W.load_library()
    assert lib.wk_ctx_create(None, None) == W.WK_EINVAL
    assert lib.wk_execute(None, None, 0, None, None) == W.WK_EINVAL
    assert lib.wk_known_to_unknown(None, None, -1, 1, 2) == W.WK_EINVAL
    assert b"null" in lib.wk_last_error()


def test_new_entry_points_reject_bad_arguments(lib_built):
    """The fork-join, batch and server entry points report bad arguments as
    statuses, whatever the device (no call here reaches the GPU)."""
    lib = W.load_library()
    h = W.wk_history()
    lib.wk_history_init(C.byref(h))
    counts = np.zeros(4, np.int64)
    p64 = counts.ctypes.data_as(C.POINTER(C.c_int64))
    assert lib.wk_history_partition(None, C.byref(h), -1, 2, p64, C.byref(h)) == W.WK_EINVAL
    assert lib.wk_history_to_device(None, C.byref(h), None, 0) == W.WK_EINVAL
    assert lib.wk_history_from_device(None, C.byref(h), None, 0, 1) == W.WK_EINVAL
    assert lib.wk_batch_set_fused(None, 1) == W.WK_EINVAL
    assert lib.wk_batch_get_fused(None) == 0
    assert lib.wk_batch_set_block_threads(None, 128) == W.WK_EINVAL
    assert lib.wk_batch_get_block_threads(None) == 0
    assert lib.wk_batch_layouts(None, 1, None, None, None) == W.WK_EINVAL
    assert lib.wk_server_cancel(None, 0) == W.WK_EINVAL
    assert lib.wk_server_inject_alloc_failure(None, 0, 1) == W.WK_EINVAL
    assert lib.wk_ctx_inject_alloc_failure(None, 1) == W.WK_EINVAL
    # a host-only context refuses device work with WK_EDEVICE
    rc = W.RCache(device=-1)
    assert lib.wk_history_partition(rc._h, C.byref(h), -1, 2, p64, C.byref(h)) == W.WK_EDEVICE
    assert lib.wk_history_to_device(rc._h, C.byref(h), None, 0) == W.WK_EDEVICE
    rc.close()


def test_no_device_is_an_error_not_a_fallback(lib_built):
    if W.device_count() > 0:
        pytest.skip("a CUDA device is present")
    with pytest.raises(W.WkError) as ei:
        W.RCache(device=0)
    assert ei.value.status == W.WK_EDEVICE


def test_graph_generator_rejects_bad_specs(lib_built):
    bad = W.graph_spec(1, 0, 3, [dict(kind=0, count=2, zipf_s=1.2, zipf_cap=8, participation=0.1)])
    with pytest.raises(W.WkError):
        W.Graph(bad)
    bad = W.graph_spec(1, 1000, 3, [dict(kind=7, count=2)])
    with pytest.raises(W.WkError):
        W.Graph(bad)


def test_batch_results_are_views_of_the_packed_array():
    """A batch's per-query tables index into one packed host array: query i
    has rows[i] rows of cols[i] columns from offset offs[i]."""
    import numpy as np
    buf = np.arange(40, dtype=np.int32)
    rows = np.array([2, 0, 3, 1], np.int64)
    cols = np.array([2, 3, 1, 4], np.int32)
    offs = np.array([0, 4, 4, 7], np.int64)
    res = W.BatchResults(buf, rows, cols, offs)
    assert len(res) == 4
    assert [t.shape for t in res] == [(2, 2), (0, 3), (3, 1), (1, 4)]
    assert res[0].tolist() == [[0, 1], [2, 3]] and res[-1].tolist() == [[7, 8, 9, 10]]
    assert [t.shape for t in res[1:3]] == [(0, 3), (3, 1)]
    assert np.shares_memory(res[2], buf)
    with pytest.raises(IndexError):
        res[4]
