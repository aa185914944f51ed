"""Fork-join across ranks (core/engine.hpp:355-395, core/gpu_engine.hpp:293-370,
core/rcache.hpp:964-1030): the split by owner and the exchange give every
rank the rows whose start vertex it owns, and the gathered result equals
the single-process one as a multiset of rows.

The multi-rank runs are gloo processes on the CPU with the oracle as each
rank's executor; the GPU tests check the device split against the same
rule and run the GPU executor on a one-rank NCCL group.
"""
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

import oracle
import wukonggpu_gb300 as W
from wukonggpu_gb300 import distributed as D
from wukonggpu_gb300 import workloads


def _split(table: np.ndarray, col: int, nparts: int):
    """The stable split by owner: (rows in owner order, rows per owner)."""
    owner = table[:, col].astype(np.uint32) % np.uint32(nparts)
    order = np.argsort(owner, kind="stable")
    return table[order], np.bincount(owner, minlength=nparts).astype(np.int64)


class OracleExecutor:
    """One rank's ops on the CPU: the oracle's step on torch CPU tensors."""

    def __init__(self, orc, torch):
        self.orc, self.torch = orc, torch

    def empty(self, n):
        return self.torch.empty(int(n), dtype=self.torch.int32)

    def counts_tensor(self, counts):
        return self.torch.as_tensor(np.asarray(counts, np.int64))

    def _np(self, table, cols):
        return table.numpy().reshape(-1, cols)

    def start(self, pattern):
        t, _ = self.orc.step(None, True, *pattern)
        return self.torch.from_numpy(np.ascontiguousarray(t, np.int32).reshape(-1)), t.shape[1]

    def partition(self, table, cols, start, nparts):
        t, counts = _split(self._np(table, cols), -start - 1, nparts)
        return self.torch.from_numpy(np.ascontiguousarray(t).reshape(-1)), counts

    def step(self, table, cols, pattern):
        t, _ = self.orc.step(self._np(table, cols), False, *pattern)
        return self.torch.from_numpy(np.ascontiguousarray(t, np.int32).reshape(-1))

    def to_numpy(self, table, cols):
        return self._np(table, cols)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, queries, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        g = W.Graph(W.spec_small())
        s, p, o = (np.array(a) for a in g.arrays())
        fj = D.ForkJoin(OracleExecutor(oracle.Oracle(s, p, o, g.num_ids), torch), dist)
        out = []
        for name, cmd in queries:
            res, per_step = fj.execute(cmd)
            out.append((name, oracle.rows_digest(res) if rank == 0 else None,
                        None if res is None else res.shape[0], per_step))
        q.put((rank, out))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_forkjoin_equals_single_process(world, small_graph, small_oracle):
    g, s, p, o = small_graph
    queries = workloads.small_queries(s, p, o)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, queries, q)) for r in range(world)]
    for pr in procs:
        pr.start()
    got = dict(q.get(timeout=600) for _ in range(world))
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    for i, (name, cmd) in enumerate(queries):
        exp, erows = small_oracle.execute(cmd)
        _, digest, nrows, per_step0 = got[0][i]
        assert digest == oracle.rows_digest(exp), name
        assert nrows == exp.shape[0], name
        # every later step's rows, summed over the ranks, are the
        # single-process counts
        assert per_step0[0] == erows[0], name
        for k in range(1, len(erows)):
            assert sum(got[r][i][3][k] for r in range(world)) == erows[k], (name, k)
        # the start runs on rank 0 only
        assert all(got[r][i][3][0] == 0 for r in range(1, world)), name


@pytest.mark.gpu
@pytest.mark.parametrize("R,C,nparts", [(0, 2, 2), (1, 1, 3), (1000, 3, 2), (70001, 4, 7), (5000, 2, 256),
                                         (300_001, 1, 8), (123_457, 9, 31), (1000, 2, 1)])
def test_device_partition_is_a_stable_split(gpu_small, R, C, nparts):
    rng = np.random.default_rng(R + C + nparts)
    table = rng.integers(0, 1 << 30, size=(R, C), dtype=np.int64).astype(np.int32)
    req = W.Request([])
    gpu_small.upload_history(req, table if R else np.zeros((0, C), np.int32))
    col = C - 1
    counts = gpu_small.partition(req, -col - 1, nparts)
    exp, ecounts = _split(table, col, nparts)
    assert list(counts) == list(ecounts)
    assert req.col_num == C and req.get_row_num() == R
    got = gpu_small.download(req)
    assert np.array_equal(got.reshape(-1, C) if R else got.reshape(0, C), exp.reshape(-1, C))


@pytest.mark.gpu
def test_device_partition_rejects_bad_arguments(gpu_small):
    req = W.Request([])
    gpu_small.upload_history(req, np.arange(12, dtype=np.int32).reshape(6, 2))
    for start, nparts in [(-3, 2), (0, 2), (-1, 0), (-1, 257)]:
        with pytest.raises(W.WkError):
            gpu_small.partition(req, start, nparts)


@pytest.mark.gpu
def test_gpu_executor_one_rank(small_graph, small_oracle, gpu_small):
    """The GPU executor through a one-rank NCCL group: the partition, the
    exchange and the gather are the multi-rank code path."""
    import torch
    import torch.distributed as dist
    g, s, p, o = small_graph
    torch.cuda.set_device(0)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(_free_port()))
    dist.init_process_group("nccl", rank=0, world_size=1)
    try:
        fj = D.ForkJoin(D.GpuExecutor(gpu_small, torch), dist)
        for name, cmd in workloads.small_queries(s, p, o):
            res, per_step = fj.execute(cmd)
            exp, erows = small_oracle.execute(cmd)
            assert oracle.rows_digest(res) == oracle.rows_digest(exp), name
            assert list(per_step) == list(erows), name
    finally:
        dist.destroy_process_group()


def _gpu_rank_main(rank, world, port, queries, q):
    """A rank with the GPU executor on the one GPU; tables cross ranks as host
    tensors over gloo, so no rank's kernels wait on another's."""
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        g = W.Graph(W.spec_small())
        rc = W.RCache(device=0)
        rc.build_store_graph(g)
        fj = D.ForkJoin(D.GpuExecutor(rc, torch, host_tables=True), dist)
        out = []
        for name, cmd in queries:
            res, per_step = fj.execute(cmd)
            out.append((name, oracle.rows_digest(res) if rank == 0 else None, per_step))
        rc.close()
        q.put((rank, out))
    finally:
        dist.destroy_process_group()


@pytest.mark.gpu
def test_gpu_executors_on_two_ranks(small_graph, small_oracle):
    """Two ranks, each with its own context and store replica on the GPU, run
    the split, the exchange (gloo, host tensors) and the steps of every query;
    the gathered rows equal the single-process result."""
    g, s, p, o = small_graph
    queries = workloads.small_queries(s, p, o)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_gpu_rank_main, args=(r, 2, port, queries, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    got = dict(q.get(timeout=600) for _ in range(2))
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    for i, (name, cmd) in enumerate(queries):
        exp, erows = small_oracle.execute(cmd)
        assert got[0][i][1] == oracle.rows_digest(exp), name
        for k in range(1, len(erows)):
            assert got[0][i][2][k] + got[1][i][2][k] == erows[k], (name, k)
