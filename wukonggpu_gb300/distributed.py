"""Fork-join execution of a query across ranks.

The reference runs a pattern where the rows' start vertices live: before a
step whose start variable is not the one the table is split by, a server
splits its table by the owner of each row's start vertex and sends every
part to its owner (Engine::need_fork_join / generate_sub_requests,
core/engine.hpp:355-395; GPU_Engine::generate_sub_query,
core/gpu_engine.hpp:293-370, with RCache::generate_sub_query,
core/rcache.hpp:964-1030); the owners run the step on their parts and the
parent merges the replies (core/gpu_engine.hpp:495-530).

Here every rank holds a replica of the store on its GPU and the split is
the device op ``wk_history_partition`` (owner = value % world size, the rule
of mymath::hash_mod); the parts move with one ``all_to_all_single`` of the
row counts and one of the rows, over NCCL between GPUs or gloo between CPU
processes.  Rank 0 runs the first pattern (an index or constant start), the
others start empty; at the end rank 0 gathers every rank's rows.  The rows
of a part keep their order, but the parts arrive in rank order, so a
result equals the single-process one as a multiset of rows.

An executor holds one rank's tables as flat int32 tensors with a column
count; ``GpuExecutor`` runs the GPU ops of an ``RCache`` on CUDA tensors, or,
with ``host_tables=True``, keeps the tables in host memory between ops (for a
group whose backend exchanges host tensors, such as gloo): each op uploads
its table, runs on the device and brings the result back.
"""
from __future__ import annotations

import numpy as np

from . import Request


def _kind(pattern, cols: int) -> str:
    """The op of a later step (GPU_Engine::execute_one_step,
    core/gpu_engine.hpp:395-467): an unbound end variable expands, a bound one
    closes a cycle, a constant end is checked."""
    end = int(pattern[3])
    if end < 0:
        return "k2u" if -end - 1 >= cols else "k2k"
    return "k2c"


class GpuExecutor:
    """One rank's ops on its GPU context; tables are CUDA int32 tensors, or
    host int32 tensors with ``host_tables=True``."""

    def __init__(self, rc, torch, host_tables: bool = False):
        self.rc, self.torch, self.host = rc, torch, host_tables
        self.device = torch.device("cpu") if host_tables else torch.device("cuda", torch.cuda.current_device())

    def empty(self, n: int):
        return self.torch.empty(int(n), dtype=self.torch.int32, device=self.device)

    def counts_tensor(self, counts):
        return self.torch.as_tensor(np.asarray(counts, np.int64), device=self.device)

    def _req(self, table, cols: int) -> Request:
        req = Request([])
        if self.host:
            self.rc.upload_history(req, table.numpy().reshape(-1, cols))
            return req
        self.torch.cuda.current_stream().synchronize()   # the collective's writes are on torch's stream
        self.rc.from_device(req, table.data_ptr(), table.numel(), cols)
        return req

    def _table(self, req: Request):
        if self.host:
            return self.torch.from_numpy(np.ascontiguousarray(self.rc.download(req)).reshape(-1))
        t = self.empty(req.hist.size)
        self.torch.cuda.current_stream().synchronize()
        self.rc.to_device(req, t.data_ptr(), t.numel())
        return t

    def start(self, pattern):
        req, _ = self.rc.execute(pattern, download=False)
        return self._table(req), req.col_num

    def partition(self, table, cols: int, start: int, nparts: int):
        req = self._req(table, cols)
        counts = self.rc.partition(req, start, nparts)
        return self._table(req), counts

    def step(self, table, cols: int, pattern):
        start, pid, d, end = (int(x) for x in pattern)
        req = self._req(table, cols)
        kind = _kind(pattern, cols)
        if kind == "k2u":
            self.rc.known_to_unknown(req, start, d, pid)
        elif kind == "k2k":
            self.rc.known_to_known(req, start, d, pid, end)
        else:
            self.rc.known_to_const(req, start, d, pid, end)
        return self._table(req)

    def to_numpy(self, table, cols: int) -> np.ndarray:
        return table.cpu().numpy().reshape(-1, max(cols, 1))


class ForkJoin:
    """Run queries across the ranks of a process group (torch.distributed)."""

    def __init__(self, executor, dist, group=None):
        self.ex, self.dist, self.group = executor, dist, group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)

    def _exchange(self, table, cols: int, start: int):
        """Send every row to the owner of its start vertex; returns this
        rank's rows (the parts of all ranks for this rank, in rank order)."""
        table, counts = self.ex.partition(table, cols, start, self.world)
        send = self.ex.counts_tensor(counts)
        recv = self.ex.counts_tensor(np.zeros(self.world, np.int64))
        self.dist.all_to_all_single(recv, send, group=self.group)
        rcounts = [int(x) for x in recv.cpu().tolist()]
        out = self.ex.empty(sum(rcounts) * cols)
        self.dist.all_to_all_single(out, table, [c * cols for c in rcounts], [int(c) * cols for c in counts],
                                    group=self.group)
        return out

    def _gather(self, table, cols: int):
        """Every rank's rows on rank 0 (in rank order); None elsewhere."""
        n = self.ex.counts_tensor([table.numel()])
        sizes = [self.ex.counts_tensor([0]) for _ in range(self.world)]
        self.dist.all_gather(sizes, n, group=self.group)
        sizes = [int(x.item()) for x in sizes]
        if self.rank != 0:
            if sizes[self.rank]:
                self.dist.send(table, dst=0, group=self.group)
            return None
        parts = [self.ex.to_numpy(table, cols)]
        for r in range(1, self.world):
            if sizes[r]:
                buf = self.ex.empty(sizes[r])
                self.dist.recv(buf, src=r, group=self.group)
                parts.append(self.ex.to_numpy(buf, cols))
        return np.concatenate(parts).reshape(-1, max(cols, 1))

    def execute(self, cmd_chains):
        """Run every pattern; returns (the result on rank 0 / None elsewhere,
        this rank's row count after every step)."""
        cmd = [int(x) for x in cmd_chains]
        pats = [cmd[i:i + 4] for i in range(0, len(cmd), 4)]
        if self.rank == 0:
            table, cols = self.ex.start(pats[0])
        else:
            table, cols = self.ex.empty(0), 1     # a start binds one column
        per_step = [table.numel() // max(cols, 1)]
        local_var = None
        for pat in pats[1:]:
            if pat[0] != local_var:               # Engine::need_fork_join: split by a new start
                table = self._exchange(table, cols, pat[0])
                local_var = pat[0]
            kind = _kind(pat, cols)
            if table.numel():
                table = self.ex.step(table, cols, pat)
            if kind == "k2u":
                cols += 1
            per_step.append(table.numel() // cols)
        return self._gather(table, cols), per_step
