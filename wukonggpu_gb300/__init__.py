"""GB300-native per-triple-pattern graph-exploration operator (Wukong+G GPU engine surface).

The compute path is ``libwkgpu.so`` (C++ host runtime + hand-written sm_103a
kernels) behind the C ABI declared in ``include/wukong_gpu.h``.  This module
is a thin ctypes mirror of the reference's GPU-engine interface:

* :class:`Request` mirrors ``request_or_reply`` (core/query.hpp:45-175):
  ``cmd_chains``, ``step``, ``col_num`` and the device history.
* :class:`RCache` mirrors ``RCache``'s ops (core/rcache.hpp:232, :417, :614,
  :811) plus the constant start of ``Engine::const_to_unknown``
  (core/engine.hpp:96-122), and :meth:`RCache.execute` mirrors
  ``GPU_Engine::execute_request`` (core/gpu_engine.hpp:471-526).

There is no CPU fallback: if the library is missing every entry point raises.
"""
from __future__ import annotations

import ctypes as C
import collections.abc
import itertools
import os
from pathlib import Path

import numpy as np

_PKG = Path(__file__).resolve().parent
_LIB_PATH = _PKG / "libwkgpu.so"

WK_OK, WK_EINVAL, WK_ENOMEM, WK_ETIMEDOUT, WK_EDEVICE, WK_ENOSTORE, WK_EOVERFLOW = 0, -1, -2, -3, -4, -5, -6
WK_ECANCELED, WK_EREJECTED = -7, -8
IN, OUT = 0, 1
PREDICATE_ID, TYPE_ID = 0, 1
VID_BASE = 1 << 17


class WkError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"[{status}] {msg}")
        self.status = status


class wk_config(C.Structure):
    _fields_ = [("device", C.c_int32), ("cache_budget_mb", C.c_int32), ("enable_prefetch", C.c_int32),
                ("reserved", C.c_int32), ("history_capacity", C.c_int64)]


class wk_history(C.Structure):
    _fields_ = [("data", C.c_void_p), ("size", C.c_int64), ("col_num", C.c_int32), ("step", C.c_int32)]


class wk_store_info(C.Structure):
    _fields_ = [("num_keys", C.c_int64), ("num_edges", C.c_int64), ("key_bytes", C.c_int64),
                ("edge_bytes", C.c_int64), ("overflow_buckets", C.c_int64), ("device_bytes", C.c_int64),
                ("num_ids", C.c_int32), ("paged", C.c_int32), ("cache_loads", C.c_int64),
                ("cache_evictions", C.c_int64), ("cache_bytes_loaded", C.c_int64), ("dense_dirs", C.c_int64),
                ("cache_requests", C.c_int64), ("cache_hits", C.c_int64), ("cache_compactions", C.c_int64)]


class wk_seg_layout(C.Structure):
    _fields_ = [("keys", C.c_int64), ("edges", C.c_int64), ("main_buckets", C.c_int32),
                ("overflow_buckets", C.c_int32), ("dense", C.c_int32 * 2), ("functional", C.c_int32 * 2),
                ("bitmap", C.c_int32 * 2), ("max_degree", C.c_int32 * 2), ("device_bytes", C.c_int64)]


class wk_op_stats(C.Structure):
    _fields_ = [("ms", C.c_double), ("ms_main", C.c_double), ("rows_in", C.c_int64), ("rows_out", C.c_int64),
                ("cols_in", C.c_int32), ("kind", C.c_int32), ("alg_bytes", C.c_int64), ("kernels", C.c_int64),
                ("span_ms", C.c_double)]


class wk_server_config(C.Structure):
    _fields_ = [("mode", C.c_int32), ("max_batch", C.c_int32), ("max_steps", C.c_int32), ("heavy_workers", C.c_int32),
                ("batch_capacity_ints", C.c_int64), ("light_budget_bytes", C.c_int64), ("plan", C.c_int32),
                ("keep_results", C.c_int32), ("batch_window_us", C.c_int32), ("pad", C.c_int32),
                ("max_request_bytes", C.c_int64)]


class wk_server_stats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("light", C.c_int64), ("heavy", C.c_int64), ("failed", C.c_int64),
                ("batches", C.c_int64), ("mean_batch", C.c_double), ("span_s", C.c_double), ("qps", C.c_double),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("light_p50_ms", C.c_double),
                ("light_p99_ms", C.c_double), ("heavy_p50_ms", C.c_double), ("heavy_p99_ms", C.c_double),
                ("rejected", C.c_int64), ("cancelled", C.c_int64)]


class wk_type_stats(C.Structure):
    _fields_ = [("completed", C.c_int64), ("failed", C.c_int64), ("qps", C.c_double), ("p50_ms", C.c_double),
                ("p99_ms", C.c_double), ("cdf_ms", C.c_double * 25)]


class wk_pred_group(C.Structure):
    _fields_ = [("kind", C.c_int32), ("count", C.c_int32), ("zipf_s", C.c_double), ("zipf_cap", C.c_int32),
                ("pad", C.c_int32), ("participation", C.c_double), ("hub_frac", C.c_double)]


class wk_graph_spec(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("n_entities", C.c_int64), ("n_classes", C.c_int32),
                ("n_groups", C.c_int32), ("groups", wk_pred_group * 4)]


_P = C.c_void_p
_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)

_SIGS = {
    "wk_config_default": (None, [C.POINTER(wk_config)]),
    "wk_ctx_create": (C.c_int, [C.POINTER(wk_config), C.POINTER(_P)]),
    "wk_ctx_destroy": (C.c_int, [_P]),
    "wk_last_error": (C.c_char_p, []),
    "wk_status_str": (C.c_char_p, [C.c_int]),
    "wk_device_count": (C.c_int, [C.POINTER(C.c_int)]),
    "wk_store_build": (C.c_int, [_P, _I32P, _I32P, _I32P, C.c_int64, C.c_int32]),
    "wk_store_build_device": (C.c_int, [_P, _I32P, _I32P, _I32P, C.c_int64, C.c_int32]),
    "wk_store_digest": (C.c_int, [_P, C.POINTER(C.c_uint64)]),
    "wk_ctx_share_store": (C.c_int, [_P, _P]),
    "wk_store_get_info": (C.c_int, [_P, C.POINTER(wk_store_info)]),
    "wk_store_get_edges": (C.c_int, [_P, C.c_int64, C.c_int32, C.c_int32, _I32P, C.c_int64, _I64P]),
    "wk_store_pred_stats": (C.c_int, [_P, C.c_int32, _I64P, _I64P, _I64P]),
    "wk_known_to_unknown": (C.c_int, [_P, C.POINTER(wk_history), C.c_int64, C.c_int32, C.c_int32]),
    "wk_known_to_known": (C.c_int, [_P, C.POINTER(wk_history), C.c_int64, C.c_int32, C.c_int32, C.c_int64]),
    "wk_known_to_const": (C.c_int, [_P, C.POINTER(wk_history), C.c_int64, C.c_int32, C.c_int32, C.c_int64]),
    "wk_index_to_unknown": (C.c_int, [_P, C.POINTER(wk_history), C.c_int32, C.c_int32]),
    "wk_const_to_unknown": (C.c_int, [_P, C.POINTER(wk_history), C.c_int64, C.c_int32, C.c_int32]),
    "wk_known_to_unknown_noalloc": (C.c_int, [_P, _P, C.c_int64, C.c_int32, C.c_int64, C.c_int32, C.c_int32, _P,
                                             C.c_int64, _I64P]),
    "wk_history_upload": (C.c_int, [_P, C.POINTER(wk_history), _I32P, C.c_int64, C.c_int32]),
    "wk_history_download": (C.c_int, [_P, C.POINTER(wk_history), _I32P, C.c_int64]),
    "wk_history_init": (None, [C.POINTER(wk_history)]),
    "wk_history_partition": (C.c_int, [_P, C.POINTER(wk_history), C.c_int64, C.c_int32, _I64P,
                                       C.POINTER(wk_history)]),
    "wk_history_to_device": (C.c_int, [_P, C.POINTER(wk_history), _P, C.c_int64]),
    "wk_history_from_device": (C.c_int, [_P, C.POINTER(wk_history), _P, C.c_int64, C.c_int32]),
    "wk_execute": (C.c_int, [_P, _I64P, C.c_int32, C.POINTER(wk_history), _I64P]),
    "wk_enable_timing": (C.c_int, [_P, C.c_int]),
    "wk_last_op_stats": (C.c_int, [_P, C.POINTER(wk_op_stats)]),
    "wk_query_op_stats": (C.c_int, [_P, C.POINTER(wk_op_stats), C.c_int32, C.POINTER(C.c_int32)]),
    "wk_kernel_launches": (C.c_int64, [_P]),
    "wk_sync": (C.c_int, [_P]),
    "wk_plan": (C.c_int, [_P, _I64P, C.c_int32, _I64P, C.POINTER(C.c_int32), C.POINTER(C.c_double),
                          C.POINTER(C.c_int32)]),
    "wk_stat_get": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32, _I64P]),
    "wk_batch_create": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int64, C.POINTER(_P)]),
    "wk_batch_destroy": (C.c_int, [_P]),
    "wk_batch_run": (C.c_int, [_P, _I64P, _I32P, C.c_int32, C.c_int32]),
    "wk_batch_launch": (C.c_int, [_P, _I64P, _I32P, C.c_int32, C.c_int32]),
    "wk_batch_ready": (C.c_int, [_P]),
    "wk_batch_wait": (C.c_int, [_P]),
    "wk_batch_result": (C.c_int, [_P, C.c_int32, _I64P, _I32P, _I64P]),
    "wk_batch_download": (C.c_int, [_P, _I32P, C.c_int64, _I64P]),
    "wk_batch_set_tuning": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_int32]),
    "wk_batch_get_tuning": (C.c_int, [_P, _I32P, _I32P, _I32P]),
    "wk_batch_set_fused": (C.c_int, [_P, C.c_int32]),
    "wk_batch_layouts": (C.c_int, [_P, C.c_int32, _I64P, _I32P, _I64P]),
    "wk_batch_autotune_forms": (C.c_int, [_P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
    "wk_batch_get_fused": (C.c_int, [_P]),
    "wk_batch_set_block_threads": (C.c_int, [_P, C.c_int32]),
    "wk_batch_get_block_threads": (C.c_int, [_P]),
    "wk_batch_autotune": (C.c_int, [_P, _I64P, _I32P, C.c_int32, C.c_int32, C.POINTER(C.c_double)]),
    "wk_batch_kernel_launches": (C.c_int64, [_P]),
    "wk_server_config_default": (None, [C.POINTER(wk_server_config)]),
    "wk_server_create": (C.c_int, [_P, C.POINTER(wk_server_config), C.POINTER(_P)]),
    "wk_server_submit": (C.c_int64, [_P, _I64P, C.c_int32, C.c_double]),
    "wk_server_start": (C.c_int, [_P]),
    "wk_server_drain": (C.c_int, [_P, C.c_double]),
    "wk_server_result": (C.c_int, [_P, C.c_int64, _I64P, _I32P, _I32P, C.c_int64, C.POINTER(C.c_double),
                                   _I32P]),
    "wk_server_get_stats": (C.c_int, [_P, C.POINTER(wk_server_stats)]),
    "wk_server_latency_cdf": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_double)]),
    "wk_server_destroy": (C.c_int, [_P]),
    "wk_server_submit_typed": (C.c_int64, [_P, _I64P, C.c_int32, C.c_double, C.c_int32]),
    "wk_server_type_stats": (C.c_int, [_P, C.c_int32, C.POINTER(wk_type_stats)]),
    "wk_server_cancel": (C.c_int, [_P, C.c_int64]),
    "wk_server_inject_alloc_failure": (C.c_int, [_P, C.c_int32, C.c_int32]),
    "wk_ctx_inject_alloc_failure": (C.c_int, [_P, C.c_int32]),
    "wk_mlp_create": (C.c_int, [_P, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(_P)]),
    "wk_mlp_destroy": (C.c_int, [_P]),
    "wk_mlp_num_params": (C.c_int64, [_P]),
    "wk_mlp_get_params": (C.c_int, [_P, C.POINTER(C.c_float), C.c_int64]),
    "wk_mlp_set_params": (C.c_int, [_P, C.POINTER(C.c_float), C.c_int64]),
    "wk_mlp_gradients": (C.c_int, [_P, C.POINTER(C.c_float), _I32P, C.POINTER(C.c_float), C.c_int32,
                                   C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "wk_mlp_train": (C.c_int, [_P, C.POINTER(C.c_float), _I32P, C.POINTER(C.c_float), C.c_int64, C.c_int32,
                               C.c_int32, C.c_float, C.c_uint64, C.POINTER(C.c_float)]),
    "wk_mlp_predict": (C.c_int, [_P, C.POINTER(C.c_float), _I32P, C.c_int64, C.POINTER(C.c_float)]),
    "wk_mlp_validate": (C.c_int, [_P, C.POINTER(C.c_float), _I32P, C.POINTER(C.c_float), C.c_int64, C.c_double,
                                  C.POINTER(C.c_double), C.POINTER(C.c_int32)]),
    "wk_mlp_is_trusted": (C.c_int, [_P]),
    "wk_featurize": (C.c_int, [_P, _I64P, C.c_int32, _I64P, C.POINTER(C.c_float), _I32P, C.POINTER(C.c_double)]),
    "wk_plan_learned": (C.c_int, [_P, _P, _I64P, C.c_int32, _I64P, C.POINTER(C.c_int32), C.POINTER(C.c_double)]),
    "wk_plan_learned_batch": (C.c_int, [_P, _P, _I64P, _I32P, C.c_int32, _I64P, _I32P]),
    "wk_set_row_limit": (C.c_int, [_P, C.c_int64]),
    "wk_timer_begin": (C.c_int, [_P]),
    "wk_timer_end": (C.c_int, [_P, C.POINTER(C.c_double)]),
    "wk_host_alloc": (C.c_int, [C.c_int64, C.POINTER(_P)]),
    "wk_host_free": (C.c_int, [_P]),
    "wk_store_seg_layout": (C.c_int, [_P, C.c_int32, C.POINTER(wk_seg_layout)]),
    "wk_graph_generate": (C.c_int, [C.POINTER(wk_graph_spec), C.c_int32, C.POINTER(_P)]),
    "wk_graph_size": (C.c_int64, [_P]),
    "wk_graph_num_ids": (C.c_int32, [_P]),
    "wk_graph_first_class": (C.c_int32, [_P]),
    "wk_graph_s": (_I32P, [_P]),
    "wk_graph_p": (_I32P, [_P]),
    "wk_graph_o": (_I32P, [_P]),
    "wk_graph_free": (None, [_P]),
    "wk_store_build_graph": (C.c_int, [_P, _P]),
}

_lib = None
_gen = None
_GEN_LIB_PATH = _PKG / "libwkgen.so"
_GEN_SIGS = {k: _SIGS[k] for k in ("wk_graph_generate", "wk_graph_size", "wk_graph_num_ids", "wk_graph_first_class",
                                   "wk_graph_s", "wk_graph_p", "wk_graph_o", "wk_graph_free", "wk_last_error")}


def lib_path() -> Path:
    return _LIB_PATH


def load_gen_library():
    """Load libwkgen.so, the seeded graph generator alone (host code, no CUDA),
    so that a process that only needs a graph -- the CPU baseline -- does not
    map the GPU library."""
    global _gen
    if _gen is not None:
        return _gen
    if not _GEN_LIB_PATH.exists():
        raise ImportError(f"{_GEN_LIB_PATH} is missing: build it with `python -m wukonggpu_gb300.build`")
    lib = C.CDLL(str(_GEN_LIB_PATH))
    for name, (res, args) in _GEN_SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _gen = lib
    return lib


def load_library():
    """Load libwkgpu.so; raises if it has not been built (no fallback)."""
    global _lib
    if _lib is not None:
        return _lib
    if not _LIB_PATH.exists():
        raise ImportError(f"{_LIB_PATH} is missing: build it with `python -m wukonggpu_gb300.build`")
    lib = C.CDLL(str(_LIB_PATH))
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def exported_symbols():
    return list(_SIGS)


def _check(status: int):
    if status != WK_OK:
        raise WkError(status, load_library().wk_last_error().decode(errors="replace"))


def _i32(a: np.ndarray):
    return a.ctypes.data_as(_I32P)


# --------------------------------------------------------------- graphs
def graph_spec(seed: int, n_entities: int, n_classes: int, groups) -> wk_graph_spec:
    sp = wk_graph_spec()
    sp.seed = seed
    sp.n_entities = n_entities
    sp.n_classes = n_classes
    sp.n_groups = len(groups)
    for i, g in enumerate(groups):
        sp.groups[i].kind = g.get("kind", 0)
        sp.groups[i].count = g["count"]
        sp.groups[i].zipf_s = g.get("zipf_s", 1.0)
        sp.groups[i].zipf_cap = g.get("zipf_cap", 1)
        sp.groups[i].participation = g.get("participation", 1.0)
        sp.groups[i].hub_frac = g.get("hub_frac", 0.01)
    return sp


def spec_small(seed: int = 20240601) -> wk_graph_spec:
    """200k entities, rdf:type with 10 classes, 15 Zipf(1.2, cap 64) predicates, ~1M triples."""
    return graph_spec(seed, 200_000, 10, [dict(kind=0, count=15, zipf_s=1.2, zipf_cap=64, participation=0.027)])


def spec_single_query(seed: int = 20240602, scale: float = 1.0) -> wk_graph_spec:
    """2M entities (x scale), 15 classes, 8 one-to-one, 16 Zipf(1.1, cap 4096), 8 many-to-one onto 1% hubs.

    About 100M triples at scale 1.0."""
    n = int(2_000_000 * scale)
    return graph_spec(seed, n, 15, [
        dict(kind=1, count=8, participation=1.0),
        dict(kind=0, count=16, zipf_s=1.1, zipf_cap=4096, participation=0.0065),
        dict(kind=2, count=8, participation=1.0, hub_frac=0.01),
    ])


def spec_serving(seed: int = 20240604, scale: float = 1.0) -> wk_graph_spec:
    """20M entities (x scale), 15 classes, 16 one-to-one, 32 Zipf(1.1, cap 4096), 16 many-to-one onto
    1% hubs: the single-query graph's degree mixes on 64 predicates.  About 1.0e9 triples at scale 1.0."""
    n = int(20_000_000 * scale)
    return graph_spec(seed, n, 15, [
        dict(kind=1, count=16, participation=1.0),
        dict(kind=0, count=32, zipf_s=1.1, zipf_cap=4096, participation=0.0017),
        dict(kind=2, count=16, participation=1.0, hub_frac=0.01),
    ])


class Graph:
    """A seeded synthetic ID-form RDF graph (owned by the library)."""

    def __init__(self, spec: wk_graph_spec, n_threads: int = 0):
        lib = load_gen_library()
        h = _P()
        st = lib.wk_graph_generate(C.byref(spec), n_threads, C.byref(h))
        if st != WK_OK:
            raise WkError(st, lib.wk_last_error().decode(errors="replace"))
        self._h = h
        self.spec = spec
        self.n = lib.wk_graph_size(h)
        self.num_ids = lib.wk_graph_num_ids(h)
        self.first_class = lib.wk_graph_first_class(h)

    def arrays(self):
        """(s, p, o) as numpy views into library memory (valid while the graph lives)."""
        lib = load_gen_library()
        out = []
        for f in (lib.wk_graph_s, lib.wk_graph_p, lib.wk_graph_o):
            ptr = f(self._h)
            out.append(np.ctypeslib.as_array(ptr, shape=(self.n,)) if self.n else np.zeros(0, np.int32))
        return tuple(out)

    def close(self):
        if getattr(self, "_h", None):
            load_gen_library().wk_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ------------------------------------------------------ request / engine
class Request:
    """Mirror of request_or_reply (core/query.hpp:45-175) for the GPU path."""

    def __init__(self, cmd_chains):
        self.cmd_chains = [int(x) for x in cmd_chains]
        if len(self.cmd_chains) % 4:
            raise ValueError("cmd_chains must hold 4 values per pattern")
        self.hist = wk_history()
        load_library().wk_history_init(C.byref(self.hist))
        self.result_table = None

    @property
    def step(self):
        return self.hist.step

    @property
    def col_num(self):
        return self.hist.col_num

    def get_row_num(self):
        return 0 if self.hist.col_num == 0 else self.hist.size // self.hist.col_num

    def is_finished(self):
        return self.hist.step * 4 >= len(self.cmd_chains)


class RCache:
    """A device context with its store: the GB300 counterpart of RCache + GPU_Engine."""

    def __init__(self, device: int = 0, cache_budget_mb: int = 0, enable_prefetch: bool = True,
                 history_capacity: int = 0):
        lib = load_library()
        cfg = wk_config()
        lib.wk_config_default(C.byref(cfg))
        cfg.device = device
        cfg.cache_budget_mb = cache_budget_mb
        cfg.enable_prefetch = 1 if enable_prefetch else 0
        cfg.history_capacity = history_capacity
        h = _P()
        _check(lib.wk_ctx_create(C.byref(cfg), C.byref(h)))
        self._h = h

    # -- store
    def build_store(self, s, p, o, num_ids: int, on_device: bool = False):
        """Build the store from ID-form triples; on_device builds the whole
        image on the GPU (wk_store_build_device; the same image)."""
        s = np.ascontiguousarray(s, np.int32)
        p = np.ascontiguousarray(p, np.int32)
        o = np.ascontiguousarray(o, np.int32)
        f = load_library().wk_store_build_device if on_device else load_library().wk_store_build
        _check(f(self._h, _i32(s), _i32(p), _i32(o), len(s), num_ids))

    def store_digest(self) -> int:
        d = C.c_uint64()
        _check(load_library().wk_store_digest(self._h, C.byref(d)))
        return d.value

    def build_store_graph(self, g: Graph):
        """The store of a generated graph, from its arrays in place (no copies)."""
        s, p, o = g.arrays()
        _check(load_library().wk_store_build(self._h, _i32(s), _i32(p), _i32(o), len(s), g.num_ids))

    def share_store(self, owner: "RCache"):
        _check(load_library().wk_ctx_share_store(self._h, owner._h))

    def store_info(self) -> dict:
        info = wk_store_info()
        _check(load_library().wk_store_get_info(self._h, C.byref(info)))
        return {f: getattr(info, f) for f, _ in info._fields_}

    def get_edges(self, vid: int, pid: int, d: int) -> np.ndarray:
        lib = load_library()
        deg = C.c_int64()
        _check(lib.wk_store_get_edges(self._h, vid, pid, d, None, 0, C.byref(deg)))
        out = np.zeros(max(deg.value, 1), np.int32)
        _check(lib.wk_store_get_edges(self._h, vid, pid, d, _i32(out), deg.value, C.byref(deg)))
        return out[:deg.value]

    def seg_layout(self, pid: int) -> dict:
        """The layout decisions of one id's segment (wk_store_seg_layout)."""
        x = wk_seg_layout()
        _check(load_library().wk_store_seg_layout(self._h, pid, C.byref(x)))
        return {"keys": x.keys, "edges": x.edges, "main_buckets": x.main_buckets,
                "overflow_buckets": x.overflow_buckets, "dense": list(x.dense), "functional": list(x.functional),
                "bitmap": list(x.bitmap), "max_degree": list(x.max_degree), "device_bytes": x.device_bytes}

    def pred_stats(self, pid: int):
        t, s, o = C.c_int64(), C.c_int64(), C.c_int64()
        _check(load_library().wk_store_pred_stats(self._h, pid, C.byref(t), C.byref(s), C.byref(o)))
        return t.value, s.value, o.value

    # -- ops (reference names and argument order)
    def known_to_unknown(self, req: Request, start: int, direction: int, predict: int):
        _check(load_library().wk_known_to_unknown(self._h, C.byref(req.hist), start, direction, predict))

    def known_to_known(self, req: Request, start: int, direction: int, predict: int, end: int):
        _check(load_library().wk_known_to_known(self._h, C.byref(req.hist), start, direction, predict, end))

    def known_to_const(self, req: Request, start: int, direction: int, predict: int, end: int):
        _check(load_library().wk_known_to_const(self._h, C.byref(req.hist), start, direction, predict, end))

    def index_to_unknown(self, req: Request, index_vertex: int, direction: int):
        _check(load_library().wk_index_to_unknown(self._h, C.byref(req.hist), index_vertex, direction))

    def const_to_unknown(self, req: Request, start: int, direction: int, predict: int):
        _check(load_library().wk_const_to_unknown(self._h, C.byref(req.hist), start, direction, predict))

    def upload_history(self, req: Request, table: np.ndarray):
        t = np.ascontiguousarray(table, np.int32)
        cols = t.shape[1] if t.ndim == 2 else 1
        _check(load_library().wk_history_upload(self._h, C.byref(req.hist), _i32(t.reshape(-1)), t.size, cols))

    # -- fork-join across ranks
    def partition(self, req: Request, start: int, nparts: int) -> np.ndarray:
        """Split req's table by owner rank (value of variable `start` modulo
        nparts) on the device; req then holds the parts one after another and
        the return value their row counts (wk_history_partition)."""
        counts = np.zeros(nparts, np.int64)
        out = wk_history()
        _check(load_library().wk_history_partition(self._h, C.byref(req.hist), start, nparts,
                                                    counts.ctypes.data_as(_I64P), C.byref(out)))
        req.hist = out
        return counts

    def to_device(self, req: Request, dst_ptr: int, cap: int):
        """Copy req's table to device memory at dst_ptr (cap int32 elements)."""
        _check(load_library().wk_history_to_device(self._h, C.byref(req.hist), C.c_void_p(dst_ptr), cap))

    def from_device(self, req: Request, src_ptr: int, size: int, cols: int):
        """Make req's table the `size` int32 elements at device address src_ptr."""
        _check(load_library().wk_history_from_device(self._h, C.byref(req.hist), C.c_void_p(src_ptr), size, cols))

    def download(self, req: Request, into: "PinnedBuffer | None" = None) -> np.ndarray:
        h = req.hist
        if into is not None and into.n >= h.size:
            _check(load_library().wk_history_download(self._h, C.byref(h), _i32(into.array), into.n))
            return into.array[:h.size].reshape(-1, max(h.col_num, 1))
        out = np.zeros(max(h.size, 1), np.int32)
        _check(load_library().wk_history_download(self._h, C.byref(h), _i32(out), out.size))
        cols = max(h.col_num, 1)
        return out[:h.size].reshape(-1, cols)

    def execute(self, cmd_chains, download: bool = True):
        """Run every pattern on the device; returns (table, per-step row counts)."""
        req = Request(cmd_chains)
        n = len(req.cmd_chains) // 4
        cc = np.asarray(req.cmd_chains, np.int64)
        rows = np.zeros(n, np.int64)
        _check(load_library().wk_execute(self._h, cc.ctypes.data_as(_I64P), n, C.byref(req.hist),
                                         rows.ctypes.data_as(_I64P)))
        req.result_table = self.download(req) if download else None
        return req, rows

    def plan(self, cmd_chains):
        """Statistics-based plan: (planned cmd_chains, estimated cost).

        None when the statistics prove the result empty; [] (cost inf) when the
        planner finds no order, as the reference does."""
        cc = np.asarray(cmd_chains, np.int64)
        n = len(cc) // 4
        out = np.zeros(4 * (n + 2), np.int64)
        n_out = C.c_int32(n + 2)
        cost = C.c_double()
        empty = C.c_int32()
        _check(load_library().wk_plan(self._h, cc.ctypes.data_as(_I64P), n, out.ctypes.data_as(_I64P),
                                      C.byref(n_out), C.byref(cost), C.byref(empty)))
        if empty.value:
            return None, 0.0
        return [int(x) for x in out[:4 * n_out.value]], cost.value

    def stat(self, which: int, a: int, b: int = 0):
        out = np.zeros(4, np.int64)
        _check(load_library().wk_stat_get(self._h, which, a, b, out.ctypes.data_as(_I64P)))
        return [int(x) for x in out] if which == 4 else int(out[0])

    def inject_alloc_failure(self, n: int):
        """The next n device-buffer reservations fail with WK_ENOMEM (host-side injection)."""
        _check(load_library().wk_ctx_inject_alloc_failure(self._h, n))

    def set_row_limit(self, max_rows: int):
        """Cap on k2u output rows (0 = none); larger steps fail with WK_EOVERFLOW."""
        _check(load_library().wk_set_row_limit(self._h, max_rows))

    def enable_timing(self, on: bool = True):
        _check(load_library().wk_enable_timing(self._h, 1 if on else 0))

    def last_op_stats(self) -> dict:
        st = wk_op_stats()
        _check(load_library().wk_last_op_stats(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    def query_op_stats(self) -> list:
        """Per-op statistics of every op of the last execute() (timing enabled)."""
        lib = load_library()
        n = C.c_int32()
        _check(lib.wk_query_op_stats(self._h, None, 0, C.byref(n)))
        arr = (wk_op_stats * max(n.value, 1))()
        _check(lib.wk_query_op_stats(self._h, arr, n.value, C.byref(n)))
        return [{f: getattr(arr[i], f) for f, _ in wk_op_stats._fields_} for i in range(n.value)]

    def kernel_launches(self) -> int:
        return load_library().wk_kernel_launches(self._h)

    def sync(self):
        _check(load_library().wk_sync(self._h))

    def timer_begin(self):
        """Record a CUDA event on the context's stream."""
        _check(load_library().wk_timer_begin(self._h))

    def timer_end(self) -> float:
        """Device milliseconds since timer_begin (synchronises the stream)."""
        ms = C.c_double()
        _check(load_library().wk_timer_end(self._h, C.byref(ms)))
        return ms.value

    def close(self):
        if getattr(self, "_h", None):
            load_library().wk_ctx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass



class BatchResults(collections.abc.Sequence):
    """The per-query tables of one batch: query i's rows are a (rows, cols)
    view into the packed host array, made when the query is indexed."""

    def __init__(self, buf: np.ndarray, rows: np.ndarray, cols: np.ndarray, offs: np.ndarray):
        self._buf, self._rows, self._cols, self._offs = buf, rows, cols, offs

    def __len__(self) -> int:
        return len(self._rows)

    def __getitem__(self, i):
        if isinstance(i, slice):
            return [self[j] for j in range(*i.indices(len(self)))]
        n = len(self._rows)
        if i < 0:
            i += n
        if not 0 <= i < n:
            raise IndexError(i)
        r, c, o = int(self._rows[i]), int(self._cols[i]), int(self._offs[i])
        return self._buf[o:o + r * c].reshape(-1, max(c, 1))


class Batch:
    """Batched execution of constant-start queries (one CUDA graph per batch shape)."""

    def __init__(self, rc: "RCache", max_queries: int = 4096, max_steps: int = 4, capacity_ints: int = 1 << 26):
        h = _P()
        _check(load_library().wk_batch_create(rc._h, max_queries, max_steps, capacity_ints, C.byref(h)))
        self._h = h
        self.rc = rc
        self.max_steps = max_steps

    @staticmethod
    def pack(queries):
        npat = np.fromiter((len(q) >> 2 for q in queries), np.int32, len(queries))
        cmd = np.fromiter(itertools.chain.from_iterable(queries), np.int64, 4 * int(npat.sum()))
        return cmd, npat

    def run(self, queries, use_graph: bool = True, packed=None):
        cmd, npat = packed if packed is not None else self.pack(queries)
        _check(load_library().wk_batch_run(self._h, cmd.ctypes.data_as(_I64P), npat.ctypes.data_as(_I32P),
                                           len(npat), 1 if use_graph else 0))
        return len(npat)

    def download(self, nq: int, into: "PinnedBuffer | None" = None) -> "BatchResults":
        """Per-query result tables of the last run: every result is copied to
        host memory (into `into` when it is large enough), and the returned
        sequence gives each query's table as a numpy view into that array."""
        lib = load_library()
        tot = C.c_int64()
        _check(lib.wk_batch_download(self._h, None, 0, C.byref(tot)))
        if into is not None and into.n >= tot.value:
            buf = into.array
        else:
            buf = np.zeros(max(tot.value, 1), np.int32)
        _check(lib.wk_batch_download(self._h, buf.ctypes.data_as(_I32P), buf.size, C.byref(tot)))
        rows = np.empty(nq, np.int64)
        cols = np.empty(nq, np.int32)
        offs = np.empty(nq, np.int64)
        _check(lib.wk_batch_layouts(self._h, nq, rows.ctypes.data_as(_I64P), cols.ctypes.data_as(_I32P),
                                    offs.ctypes.data_as(_I64P)))
        return BatchResults(buf, rows, cols, offs)

    def set_tuning(self, blocks_per_sm: int, rows_per_warp: int, split_ints: int):
        _check(load_library().wk_batch_set_tuning(self._h, blocks_per_sm, rows_per_warp, split_ints))

    def tuning(self):
        a, b, c = C.c_int32(), C.c_int32(), C.c_int32()
        _check(load_library().wk_batch_get_tuning(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def set_fused(self, fused: bool):
        """One cooperative kernel per step (True) or three kernels (False)."""
        _check(load_library().wk_batch_set_fused(self._h, 1 if fused else 0))

    def fused(self) -> bool:
        return load_library().wk_batch_get_fused(self._h) == 1

    def set_block_threads(self, threads: int):
        """Threads per block of the step kernels: 128 or 256."""
        _check(load_library().wk_batch_set_block_threads(self._h, threads))

    def block_threads(self) -> int:
        return load_library().wk_batch_get_block_threads(self._h)

    def autotune(self, queries, reps: int = 3) -> float:
        cmd, npat = self.pack(queries)
        ms = C.c_double()
        _check(load_library().wk_batch_autotune(self._h, cmd.ctypes.data_as(_I64P), npat.ctypes.data_as(_I32P),
                                                len(npat), reps, C.byref(ms)))
        return ms.value

    def kernel_launches(self) -> int:
        return load_library().wk_batch_kernel_launches(self._h)

    def autotune_forms(self):
        """The last autotune's best ms for three kernels per step and for one
        kernel per step (None where that form did not run)."""
        a, b = C.c_double(), C.c_double()
        _check(load_library().wk_batch_autotune_forms(self._h, C.byref(a), C.byref(b)))
        return (a.value if a.value >= 0 else None), (b.value if b.value >= 0 else None)

    def close(self):
        if getattr(self, "_h", None):
            load_library().wk_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_F32P = C.POINTER(C.c_float)

N_FEATURES = 48


class Estimator:
    """The learned cardinality estimator (BF16 tensor-core MLP) of a store."""

    def __init__(self, rc: "RCache", n_ids: int, max_batch: int = 4096, seed: int = 1):
        h = _P()
        _check(load_library().wk_mlp_create(rc._h, n_ids, max_batch, seed, C.byref(h)))
        self._h = h
        self.rc = rc
        self.n_ids = n_ids
        self.max_batch = max_batch

    def num_params(self) -> int:
        return load_library().wk_mlp_num_params(self._h)

    def get_params(self) -> np.ndarray:
        out = np.zeros(self.num_params(), np.float32)
        _check(load_library().wk_mlp_get_params(self._h, out.ctypes.data_as(_F32P), out.size))
        return out

    def set_params(self, p: np.ndarray):
        p = np.ascontiguousarray(p, np.float32)
        _check(load_library().wk_mlp_set_params(self._h, p.ctypes.data_as(_F32P), p.size))

    def gradients(self, feats, pids, target):
        f = np.ascontiguousarray(feats, np.float32)
        pp = np.ascontiguousarray(pids, np.int32)
        t = np.ascontiguousarray(target, np.float32)
        g = np.zeros(self.num_params(), np.float32)
        loss = C.c_float()
        _check(load_library().wk_mlp_gradients(self._h, f.ctypes.data_as(_F32P), pp.ctypes.data_as(_I32P),
                                               t.ctypes.data_as(_F32P), len(t), g.ctypes.data_as(_F32P),
                                               C.byref(loss)))
        return g, loss.value

    def train(self, feats, pids, target, epochs: int = 10, batch: int = 1024, lr: float = 1e-3, seed: int = 0):
        f = np.ascontiguousarray(feats, np.float32)
        pp = np.ascontiguousarray(pids, np.int32)
        t = np.ascontiguousarray(target, np.float32)
        loss = C.c_float()
        _check(load_library().wk_mlp_train(self._h, f.ctypes.data_as(_F32P), pp.ctypes.data_as(_I32P),
                                           t.ctypes.data_as(_F32P), len(t), epochs, batch, lr, seed, C.byref(loss)))
        return loss.value

    def predict(self, feats, pids) -> np.ndarray:
        f = np.ascontiguousarray(feats, np.float32)
        pp = np.ascontiguousarray(pids, np.int32)
        out = np.zeros(len(pp), np.float32)
        _check(load_library().wk_mlp_predict(self._h, f.ctypes.data_as(_F32P), pp.ctypes.data_as(_I32P), len(pp),
                                             out.ctypes.data_as(_F32P)))
        return out

    def validate(self, feats, pids, target, qerror_bound: float):
        """Held-out check: (p95 q-error, trusted).  An untrusted model makes the
        learned planners return the statistics planner's plans."""
        f = np.ascontiguousarray(feats, np.float32)
        pp = np.ascontiguousarray(pids, np.int32)
        t = np.ascontiguousarray(target, np.float32)
        p95 = C.c_double()
        ok = C.c_int32()
        _check(load_library().wk_mlp_validate(self._h, f.ctypes.data_as(_F32P), pp.ctypes.data_as(_I32P),
                                              t.ctypes.data_as(_F32P), len(t), float(qerror_bound), C.byref(p95),
                                              C.byref(ok)))
        return p95.value, bool(ok.value)

    @property
    def trusted(self) -> bool:
        return bool(load_library().wk_mlp_is_trusted(self._h))

    def plan(self, cmd_chains):
        cc = np.asarray(cmd_chains, np.int64)
        n = len(cc) // 4
        out = np.zeros(4 * (n + 2), np.int64)
        n_out = C.c_int32(n + 2)
        est = C.c_double()
        _check(load_library().wk_plan_learned(self.rc._h, self._h, cc.ctypes.data_as(_I64P), n,
                                              out.ctypes.data_as(_I64P), C.byref(n_out), C.byref(est)))
        return [int(x) for x in out[:4 * n_out.value]], est.value

    def plan_many(self, queries):
        """Learned plans of many BGPs at once ([] where no executable order exists)."""
        cmd = np.asarray([x for q in queries for x in q], np.int64)
        n_in = np.asarray([len(q) // 4 for q in queries], np.int32)
        out = np.zeros(int(4 * (n_in.sum() + len(queries))), np.int64)
        n_out = np.zeros(len(queries), np.int32)
        _check(load_library().wk_plan_learned_batch(self.rc._h, self._h, cmd.ctypes.data_as(_I64P),
                                                    n_in.ctypes.data_as(_I32P), len(queries),
                                                    out.ctypes.data_as(_I64P), n_out.ctypes.data_as(_I32P)))
        res, at = [], 0
        for k in n_out:
            res.append([int(x) for x in out[at:at + 4 * k]])
            at += 4 * int(k)
        return res

    def close(self):
        if getattr(self, "_h", None):
            load_library().wk_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def featurize(rc: "RCache", plan, true_rows=None):
    """(features [n x 48] float32, embedding ids [n], chained statistics estimates [n])."""
    cc = np.asarray(plan, np.int64)
    n = len(cc) // 4
    f = np.zeros((n, N_FEATURES), np.float32)
    p = np.zeros(n, np.int32)
    est = np.zeros(n, np.float64)
    tr = None if true_rows is None else np.ascontiguousarray(true_rows, np.int64)
    _check(load_library().wk_featurize(rc._h, cc.ctypes.data_as(_I64P), n,
                                       tr.ctypes.data_as(_I64P) if tr is not None else None,
                                       f.ctypes.data_as(_F32P), p.ctypes.data_as(_I32P),
                                       est.ctypes.data_as(C.POINTER(C.c_double))))
    return f, p, est


class Server:
    """The request loop (open-loop arrivals, continuous batching, overlap)."""

    def __init__(self, rc: "RCache", **kw):
        lib = load_library()
        cfg = wk_server_config()
        lib.wk_server_config_default(C.byref(cfg))
        for k, v in kw.items():
            setattr(cfg, k, v)
        h = _P()
        _check(lib.wk_server_create(rc._h, C.byref(cfg), C.byref(h)))
        self._h = h
        self.cfg = cfg

    def submit(self, cmd_chains, arrival_s: float = 0.0, qtype: int = -1) -> int:
        """Queue a request arriving `arrival_s` after start; `qtype` tags it with
        its template's index in a weighted mix (per-type statistics)."""
        cc = np.asarray(cmd_chains, np.int64)
        rid = load_library().wk_server_submit_typed(self._h, cc.ctypes.data_as(_I64P), len(cc) // 4, arrival_s,
                                                    qtype)
        if rid < 0:
            _check(int(rid))
        return rid

    def finished(self, rid: int) -> bool:
        """Whether the request has completed (run, failed, refused or cancelled)."""
        rows, cols = C.c_int64(), C.c_int32()
        return load_library().wk_server_result(self._h, rid, C.byref(rows), C.byref(cols), None, 0, None,
                                               None) == WK_OK

    def cancel(self, rid: int) -> bool:
        """Cancel a request that has not started; False when it already runs or finished."""
        return load_library().wk_server_cancel(self._h, rid) == WK_OK

    def type_stats(self, qtype: int) -> dict:
        """The reference Logger's statistics of one request type."""
        st = wk_type_stats()
        _check(load_library().wk_server_type_stats(self._h, qtype, C.byref(st)))
        return {"completed": st.completed, "failed": st.failed, "qps": st.qps, "p50_ms": st.p50_ms,
                "p99_ms": st.p99_ms, "cdf_ms": list(st.cdf_ms)}

    def inject_alloc_failure(self, worker: int, n: int):
        """The next n buffer reservations of a worker context fail with WK_ENOMEM (host-side injection)."""
        _check(load_library().wk_server_inject_alloc_failure(self._h, worker, n))

    def start(self):
        _check(load_library().wk_server_start(self._h))

    def drain(self, timeout_s: float = 600.0):
        _check(load_library().wk_server_drain(self._h, timeout_s))

    def result(self, rid: int, fetch: bool = True):
        """(table or None, latency seconds, status)."""
        lib = load_library()
        rows, cols, lat, st = C.c_int64(), C.c_int32(), C.c_double(), C.c_int32()
        _check(lib.wk_server_result(self._h, rid, C.byref(rows), C.byref(cols), None, 0, C.byref(lat), C.byref(st)))
        if not fetch:
            return None, lat.value, st.value
        out = np.zeros(max(rows.value * cols.value, 1), np.int32)
        _check(lib.wk_server_result(self._h, rid, C.byref(rows), C.byref(cols), out.ctypes.data_as(_I32P), out.size,
                                    C.byref(lat), C.byref(st)))
        return out[:rows.value * cols.value].reshape(rows.value, max(cols.value, 1)), lat.value, st.value

    def stats(self) -> dict:
        st = wk_server_stats()
        _check(load_library().wk_server_get_stats(self._h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in st._fields_}

    CDF_RATES = [0.01] + [0.05 * i for i in range(1, 20)] + [0.95 + 0.01 * i for i in range(1, 6)]

    def latency_cdf(self, cls: str = "all") -> list:
        """The reference Logger's 25-point latency CDF (ms) at CDF_RATES, of all,
        light or heavy requests."""
        out = (C.c_double * 25)()
        _check(load_library().wk_server_latency_cdf(self._h, {"all": 0, "light": 1, "heavy": 2}[cls], out))
        return list(out)

    def close(self):
        if getattr(self, "_h", None):
            load_library().wk_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def poisson_arrivals(n: int, rate_qps: float, seed: int = 0) -> np.ndarray:
    """Open-loop Poisson arrival times (seconds) of n requests at the given rate."""
    rng = np.random.default_rng(seed)
    return np.cumsum(rng.exponential(1.0 / rate_qps, size=n))


class PinnedBuffer:
    """Page-locked host int32 buffer (for host<->device history transfers)."""

    def __init__(self, n_int32: int):
        p = _P()
        _check(load_library().wk_host_alloc(max(n_int32, 1) * 4, C.byref(p)))
        self._p = p
        self.n = max(n_int32, 1)
        self.array = np.ctypeslib.as_array(C.cast(p, _I32P), shape=(self.n,))

    def close(self):
        if getattr(self, "_p", None):
            self.array = None
            load_library().wk_host_free(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def device_count() -> int:
    n = C.c_int()
    st = load_library().wk_device_count(C.byref(n))
    return n.value if st == WK_OK else 0


def canonical_rows(table: np.ndarray) -> np.ndarray:
    """Rows sorted lexicographically (the canonical order used for comparisons)."""
    t = np.asarray(table)
    if t.ndim != 2 or t.shape[0] == 0:
        return t
    return t[np.lexsort(t.T[::-1])]
