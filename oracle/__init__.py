"""CPU oracle for the per-pattern operator -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg use this package, and only as the checker / the timed CPU baseline.  The
product (``wukonggpu_gb300``) never imports it.

* :class:`Oracle` wraps ``_build/liboracle.so``, the plain-C restatement of
  the reference store and CPU engine (``wk_oracle.c``).
* :class:`RefStore` wraps ``_ref/libwkref.so``, the reference's own
  ``core/gstore.hpp`` compiled in place (only where the reference sources are
  present); it pins the restatement.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libwkref.so"
# The reference sources, for the harness that pins the restatement.  Only the
# environment names them: without WK_REFERENCE_DIR the harness is not built
# and the tests that need it skip.
REF_SRC = Path(os.environ["WK_REFERENCE_DIR"]) if os.environ.get("WK_REFERENCE_DIR") else None

_I32P = C.POINTER(C.c_int32)
_I64P = C.POINTER(C.c_int64)


class orc_table(C.Structure):
    _fields_ = [("data", _I32P), ("rows", C.c_int64), ("cols", C.c_int32), ("pad", C.c_int32)]


def build(with_ref: bool = True) -> None:
    """Compile the C restatement, and the reference harness when the sources exist."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    if with_ref and REF_SRC is not None and (REF_SRC / "core" / "gstore.hpp").exists():
        subprocess.run(["make", "-s", "-C", str(HERE), "ref", f"REF={REF_SRC}"], check=True)


_lib = None
_ref = None


def _load():
    global _lib
    if _lib is None:
        if not LIB.exists():
            build(with_ref=False)
        lib = C.CDLL(str(LIB))
        lib.orc_build.restype = C.c_void_p
        lib.orc_build.argtypes = [_I32P, _I32P, _I32P, C.c_int64, C.c_int32]
        lib.orc_free.argtypes = [C.c_void_p]
        lib.orc_get_edges.restype = C.c_int64
        lib.orc_get_edges.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.POINTER(_I32P)]
        lib.orc_num_keys.restype = C.c_int64
        lib.orc_num_keys.argtypes = [C.c_void_p]
        lib.orc_digest.restype = C.c_uint64
        lib.orc_digest.argtypes = [C.c_void_p, _I64P, _I64P]
        lib.orc_key_at.restype = C.c_int64
        lib.orc_key_at.argtypes = [C.c_void_p, C.c_int64, _I64P, _I32P, _I32P]
        lib.orc_step.restype = C.c_int
        lib.orc_step.argtypes = [C.c_void_p, C.POINTER(orc_table), C.c_int, C.c_int64, C.c_int64, C.c_int64,
                                 C.c_int64, _I64P]
        lib.orc_execute.restype = C.c_int
        lib.orc_execute.argtypes = [C.c_void_p, _I64P, C.c_int32, C.c_int32, C.POINTER(orc_table), _I64P]
        lib.orc_table_free.argtypes = [C.POINTER(orc_table)]
        lib.orc_table_set.restype = C.c_int
        lib.orc_table_set.argtypes = [C.POINTER(orc_table), _I32P, C.c_int64, C.c_int32]
        lib.orc_pred_stats.argtypes = [C.c_void_p, C.c_int32, _I64P, _I64P, _I64P]
        lib.orc_rows_digest.restype = C.c_uint64
        lib.orc_rows_digest.argtypes = [_I32P, C.c_int64, C.c_int32, C.c_int32]
        _lib = lib
    return _lib


def _table_to_numpy(t: orc_table) -> np.ndarray:
    if t.rows == 0 or t.cols == 0:
        return np.zeros((0, max(t.cols, 1)), np.int32)
    return np.ctypeslib.as_array(t.data, shape=(t.rows * t.cols,)).copy().reshape(t.rows, t.cols)


def _i32(a):
    return np.ascontiguousarray(a, np.int32)


class Oracle:
    """The C restatement of the reference store + CPU engine."""

    def __init__(self, s, p, o, num_ids: int):
        lib = _load()
        s, p, o = _i32(s), _i32(p), _i32(o)
        self._h = lib.orc_build(s.ctypes.data_as(_I32P), p.ctypes.data_as(_I32P), o.ctypes.data_as(_I32P),
                                len(s), num_ids)
        if not self._h:
            raise RuntimeError("oracle store build failed")
        self.num_ids = num_ids

    def get_edges(self, vid: int, pid: int, d: int) -> np.ndarray:
        ptr = _I32P()
        n = _load().orc_get_edges(self._h, vid, pid, d, C.byref(ptr))
        return np.ctypeslib.as_array(ptr, shape=(n,)).copy() if n else np.zeros(0, np.int32)

    def num_keys(self) -> int:
        return _load().orc_num_keys(self._h)

    def digest(self):
        """(order-independent content digest, keys, edge entries)"""
        k, e = C.c_int64(), C.c_int64()
        d = _load().orc_digest(self._h, C.byref(k), C.byref(e))
        return int(d), k.value, e.value

    def keys(self):
        """All stored keys as (vid, pid, dir) tuples."""
        lib = _load()
        out, cur = [], 0
        vid, pid, d = C.c_int64(), C.c_int32(), C.c_int32()
        while True:
            cur = lib.orc_key_at(self._h, cur, C.byref(vid), C.byref(pid), C.byref(d))
            if cur < 0:
                break
            out.append((vid.value, pid.value, d.value))
            cur += 1
        return out

    def step(self, table: np.ndarray | None, is_first: bool, start, pid, d, end):
        """One pattern; returns (new table, linear-scan entries for k2k/k2c)."""
        lib = _load()
        t = orc_table()
        if table is not None:
            tb = _i32(table)
            cols = tb.shape[1] if tb.ndim == 2 else 0
            lib.orc_table_set(C.byref(t), tb.ctypes.data_as(_I32P), tb.shape[0] if cols else 0, cols)
        sc = C.c_int64()
        rc = lib.orc_step(self._h, C.byref(t), 1 if is_first else 0, start, pid, d, end, C.byref(sc))
        if rc != 0:
            lib.orc_table_free(C.byref(t))
            raise ValueError("oracle: unsupported pattern")
        out = _table_to_numpy(t)
        lib.orc_table_free(C.byref(t))
        return out, sc.value

    def execute(self, cmd_chains, nthreads: int = 1):
        lib = _load()
        cc = np.asarray(cmd_chains, np.int64)
        n = len(cc) // 4
        t = orc_table()
        rows = np.zeros(n, np.int64)
        rc = lib.orc_execute(self._h, cc.ctypes.data_as(_I64P), n, nthreads, C.byref(t), rows.ctypes.data_as(_I64P))
        if rc != 0:
            lib.orc_table_free(C.byref(t))
            raise ValueError("oracle: query failed")
        out = _table_to_numpy(t)
        lib.orc_table_free(C.byref(t))
        return out, rows

    def pred_stats(self, pid: int):
        t, s, o = C.c_int64(), C.c_int64(), C.c_int64()
        _load().orc_pred_stats(self._h, pid, C.byref(t), C.byref(s), C.byref(o))
        return t.value, s.value, o.value

    def close(self):
        if getattr(self, "_h", None):
            _load().orc_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def ref_available() -> bool:
    return REF_LIB.exists()


def _load_ref():
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            raise FileNotFoundError(f"{REF_LIB} not built (needs the reference sources)")
        lib = C.CDLL(str(REF_LIB))
        lib.ref_build.restype = C.c_void_p
        lib.ref_build.argtypes = [_I32P, _I32P, _I32P, C.c_int64, C.c_int32, C.c_int32, C.c_int32]
        lib.ref_free.argtypes = [C.c_void_p]
        lib.ref_get_edges.restype = C.c_int64
        lib.ref_get_edges.argtypes = [C.c_void_p, C.c_int64, C.c_int32, C.c_int32, _I32P, C.c_int64]
        lib.ref_next_key.restype = C.c_int64
        lib.ref_next_key.argtypes = [C.c_void_p, C.c_int64, _I64P, _I32P, _I32P, _I64P]
        lib.ref_execute.restype = C.c_int
        lib.ref_execute.argtypes = [C.c_void_p, _I64P, C.c_int32, C.POINTER(_I32P), _I64P, C.POINTER(C.c_int32),
                                    _I64P]
        lib.ref_free_table.argtypes = [_I32P]
        lib.ref_digest.restype = C.c_uint64
        lib.ref_digest.argtypes = [C.c_void_p, _I64P, _I64P]
        lib.ref_stats.restype = C.c_void_p
        lib.ref_stats.argtypes = [C.c_void_p]
        lib.ref_stats_free.argtypes = [C.c_void_p]
        lib.ref_stat_get.restype = C.c_int
        lib.ref_stat_get.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, _I64P]
        lib.ref_plan.restype = C.c_int
        lib.ref_plan.argtypes = [C.c_void_p, _I64P, C.c_int32, _I64P, C.POINTER(C.c_int32)]
        _ref = lib
    return _ref


class RefStore:
    """The reference's own GStore (core/gstore.hpp), built by the reference loader's steps."""

    def __init__(self, s, p, o, num_ids: int, keys_million: int = 4, memstore_mb: int = 512):
        lib = _load_ref()
        s, p, o = _i32(s), _i32(p), _i32(o)
        self._h = lib.ref_build(s.ctypes.data_as(_I32P), p.ctypes.data_as(_I32P), o.ctypes.data_as(_I32P),
                                len(s), num_ids, keys_million, memstore_mb)

    def get_edges(self, vid: int, pid: int, d: int) -> np.ndarray:
        lib = _load_ref()
        n = lib.ref_get_edges(self._h, vid, pid, d, None, 0)
        out = np.zeros(max(n, 1), np.int32)
        lib.ref_get_edges(self._h, vid, pid, d, out.ctypes.data_as(_I32P), n)
        return out[:n]

    def digest(self):
        k, e = C.c_int64(), C.c_int64()
        d = _load_ref().ref_digest(self._h, C.byref(k), C.byref(e))
        return int(d), k.value, e.value

    def keys(self):
        lib = _load_ref()
        out, cur = [], 0
        vid, pid, d, deg = C.c_int64(), C.c_int32(), C.c_int32(), C.c_int64()
        while True:
            cur = lib.ref_next_key(self._h, cur, C.byref(vid), C.byref(pid), C.byref(d), C.byref(deg))
            if cur < 0:
                break
            out.append((vid.value, pid.value, d.value, deg.value))
            cur += 1
        return out

    def execute(self, cmd_chains):
        lib = _load_ref()
        cc = np.asarray(cmd_chains, np.int64)
        n = len(cc) // 4
        ptr, rows, cols = _I32P(), C.c_int64(), C.c_int32()
        step_rows = np.zeros(n, np.int64)
        rc = lib.ref_execute(self._h, cc.ctypes.data_as(_I64P), n, C.byref(ptr), C.byref(rows), C.byref(cols),
                             step_rows.ctypes.data_as(_I64P))
        if rc != 0:
            raise ValueError("reference harness: unsupported pattern")
        r, c = rows.value, cols.value
        out = np.ctypeslib.as_array(ptr, shape=(max(r * c, 1),))[:r * c].copy().reshape(r, max(c, 1))
        lib.ref_free_table(ptr)
        return out, step_rows

    def stats(self):
        """The reference statistics (generate_statistic + one-server gather)."""
        if getattr(self, "_st", None) is None:
            self._st = _load_ref().ref_stats(self._h)
        return self._st

    def stat(self, which: int, a: int, b: int = 0):
        out = np.zeros(4, np.int64)
        _load_ref().ref_stat_get(self.stats(), which, a, b, out.ctypes.data_as(_I64P))
        return [int(x) for x in out] if which == 4 else int(out[0])

    def plan(self, cmd_chains):
        """Planner::generate_plan of the reference: (plan or None when empty)."""
        cc = np.asarray(cmd_chains, np.int64)
        n = len(cc) // 4
        out = np.zeros(4 * (n + 2), np.int64)
        n_out = C.c_int32(n + 2)
        rc = _load_ref().ref_plan(self.stats(), cc.ctypes.data_as(_I64P), n, out.ctypes.data_as(_I64P),
                                  C.byref(n_out))
        if rc == 1:
            return None
        if rc != 0:
            raise ValueError("reference planner: output too long")
        return [int(x) for x in out[:4 * n_out.value]]

    def close(self):
        if getattr(self, "_st", None):
            _load_ref().ref_stats_free(self._st)
            self._st = None
        if getattr(self, "_h", None):
            _load_ref().ref_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def rows_digest(table: np.ndarray, nthreads: int = 1) -> tuple[int, int]:
    """(rows, order-independent digest) of a 2-D int32 table: equal for two
    tables holding the same rows in any order (wk_oracle.c, orc_rows_digest)."""
    t = np.ascontiguousarray(table, np.int32)
    if t.ndim != 2 or t.shape[0] == 0:
        return (0, 0)
    d = _load().orc_rows_digest(t.ctypes.data_as(_I32P), t.shape[0], t.shape[1], max(1, nthreads))
    return (int(t.shape[0]), int(d))


def canonical(table: np.ndarray) -> np.ndarray:
    t = np.asarray(table)
    if t.ndim != 2 or t.shape[0] == 0:
        return t
    return t[np.lexsort(t.T[::-1])]
