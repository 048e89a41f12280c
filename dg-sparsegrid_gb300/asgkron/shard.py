"""Row-sharded apply_A across ranks (one GPU per rank).

y = A f is sharded by output element (rows of the pair list), contiguous ranges balanced by
the work per row.  A rank holds the operators, the element table and the f blocks of its own
rows.  Its plan is a row-slice plan (``Plan.create(..., rows=(r0, r1))``, asg_plan_create_ex):
output y holds the rank's rows only, and the input f holds those rows followed by the halo --
the other elements the rows' work entries read after structure detection.  One exchange per
apply brings the halo blocks from the ranks that own them (an all-to-all of exactly those
blocks, into buffers allocated once); then each rank computes its rows with no further
communication and y stays sharded.  This is the one exchange step the path has (apply_A.m
reads column elements of f for every row, apply_A.m:125-131).

Nothing here launches kernels itself: the per-rank compute is any object with ``apply(f) -> y``
on the ranks' tensors (a row-slice Plan on GPUs; a CPU stand-in in the gloo tests).
"""
import numpy as np


def partition_rows(row_cost, nparts):
    """Contiguous row ranges [(r0, r1), ...] whose summed costs are as even as a prefix split
    allows: range k ends at the first row where the running cost reaches (k+1)/nparts of the
    total.  Costs are per-row work (listed pairs, or entries)."""
    cost = np.asarray(row_cost, dtype=np.float64)
    n = cost.size
    if nparts < 1:
        raise ValueError("partition_rows: nparts=%d" % nparts)
    csum = np.concatenate([[0.0], np.cumsum(cost)])
    total = csum[-1]
    bounds = [0]
    for k in range(1, nparts):
        target = total * k / nparts
        r = int(np.searchsorted(csum, target, side="left"))
        bounds.append(min(max(r, bounds[-1]), n))
    bounds.append(n)
    return [(bounds[k], bounds[k + 1]) for k in range(nparts)]


def row_plan(term_mats, idx1d, deg, rows, pairs=None, index_base=1, **kw):
    """Row-slice plan over rows [r0, r1) of the table (columns: any element; ``pairs`` as in
    Plan.create, index_base for its column ids).  Its f is the rows' blocks followed by
    ``plan.halo()``'s, its y the rows' blocks."""
    from .api import Plan

    return Plan.create(term_mats, idx1d, deg, pairs=pairs, index_base=index_base, rows=rows, **kw)


def exchange_lists(ranges, halos, rank):
    """Static halo exchange of one rank: for every peer q, the local element offsets (within
    this rank's range) it sends to q, and how many halo elements it receives from q.  halos[q]
    holds rank q's halo as 0-based table ids in ascending order, so the blocks from each owner
    arrive contiguously and in halo order."""
    r0, r1 = ranges[rank]
    send = []
    recv = []
    mine = np.asarray(halos[rank], dtype=np.int64)
    for q, (q0, q1) in enumerate(ranges):
        h = np.asarray(halos[q], dtype=np.int64)
        send.append(h[(h >= r0) & (h < r1)] - r0 if q != rank else np.zeros(0, dtype=np.int64))
        recv.append(int(((mine >= q0) & (mine < q1)).sum()) if q != rank else 0)
    owned = sum(recv)
    if owned != mine.size:
        raise ValueError("exchange_lists: %d of %d halo elements lie in no rank's range" % (owned, mine.size))
    return send, recv


class ShardedApply:
    """y_local = (A f)[rows of this rank] from f_local = f[rows of this rank].

    plan: this rank's row-slice plan (row_plan), or any object with apply(f) -> y on the ranks'
    tensors; ranges: every rank's row range (partition_rows); block: values per element
    (deg^d); halo: this rank's halo as 0-based table ids in ascending order (default
    plan.halo() minus index_base); group: the torch.distributed process group (None = the
    default group)."""

    def __init__(self, plan, ranges, block, halo=None, index_base=1, group=None):
        import torch
        import torch.distributed as dist

        self.plan = plan
        self.ranges = list(ranges)
        self.block = int(block)
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        if len(self.ranges) != self.world:
            raise ValueError("ShardedApply: %d ranges for %d ranks" % (len(self.ranges), self.world))
        if halo is None:
            halo = np.asarray(plan.halo(), dtype=np.int64) - index_base
        halo = np.asarray(halo, dtype=np.int64)
        if halo.size > 1 and np.any(np.diff(halo) <= 0):
            raise ValueError("ShardedApply: halo ids must ascend")
        halos = [None] * self.world
        dist.all_gather_object(halos, halo.tolist(), group=group)  # once, at set-up
        send, recv = exchange_lists(self.ranges, halos, self.rank)
        self.halo = halo
        self.send_counts = [int(s.size) * self.block for s in send]
        self.recv_counts = [c * self.block for c in recv]
        self._send_idx = np.concatenate(send) if send else np.zeros(0, dtype=np.int64)
        self._bufs = {}
        r0, r1 = self.ranges[self.rank]
        self.n_rows = r1 - r0
        self.torch = torch

    def _buffers(self, like):
        """f (rows + halo) and send buffers for this dtype/device, allocated once."""
        key = (like.dtype, like.device)
        if key not in self._bufs:
            t = self.torch
            f_all = t.empty((self.n_rows + self.halo.size) * self.block, dtype=like.dtype, device=like.device)
            send = t.empty(sum(self.send_counts), dtype=like.dtype, device=like.device)
            idx = t.from_numpy(self._send_idx).to(like.device)
            self._bufs[key] = (f_all, send, idx)
        return self._bufs[key]

    def gather_f(self, f_local):
        """The rank's input: its rows' blocks followed by the halo blocks from their owners (one
        all-to-all of exactly the halo blocks).  Returns a buffer reused by the next call."""
        import torch.distributed as dist

        if self.halo.size == 0 and self.world == 1:
            return f_local  # one rank holding every row: its rows are the whole input
        f_all, send, idx = self._buffers(f_local)
        nb = self.n_rows * self.block
        f_all[:nb].copy_(f_local)
        if self.world > 1:
            if idx.numel():
                self.torch.index_select(f_local.view(-1, self.block), 0, idx, out=send.view(-1, self.block))
            dist.all_to_all_single(f_all[nb:], send, self.recv_counts, self.send_counts, group=self.group)
        return f_all

    def apply(self, f_local, y=None):
        r0, r1 = self.ranges[self.rank]
        if f_local.numel() != (r1 - r0) * self.block:
            raise ValueError("ShardedApply: rank %d holds %d values, expected %d"
                             % (self.rank, f_local.numel(), (r1 - r0) * self.block))
        f = self.gather_f(f_local)
        return self.plan.apply(f) if y is None else self.plan.apply(f, y)
