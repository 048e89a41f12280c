"""Row-sharded apply_A across ranks (one GPU per rank).

y = A f is sharded by output element (rows of the pair list), contiguous ranges balanced by
the listed pairs per row.  Every rank holds the operators and the element table (a few MB)
and the f values of its own rows; one all-gather per apply assembles f, after which each
rank computes its rows with no further communication and y stays sharded.  This is the one
exchange step the path has (apply_A.m reads every column element of f for every row).

Nothing here launches kernels itself: the per-rank compute is a ``Plan`` built over the
rank's rows (``row_plan``), so the same code runs over NCCL on GPUs and over gloo on CPU
ranks in the tests.
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


def row_pairs(num_elems, rows, pairs=None):
    """CSR pair list holding only rows [r0, r1) of the full list (all pairs when pairs is None);
    the other rows are empty, so a plan built from it writes zeros there."""
    r0, r1 = rows
    rp = np.zeros(num_elems + 1, dtype=np.int64)
    if pairs is None:
        rp[r0 + 1:r1 + 1] = num_elems
        cols = np.tile(np.arange(num_elems, dtype=np.int32), r1 - r0)
    else:
        prp, pcl = np.asarray(pairs[0], dtype=np.int64), np.asarray(pairs[1], dtype=np.int32)
        rp[r0 + 1:r1 + 1] = prp[r0 + 1:r1 + 1] - prp[r0:r1]
        cols = pcl[prp[r0]:prp[r1]].copy()
    return np.cumsum(rp), cols


def row_plan(term_mats, idx1d, deg, rows, pairs=None, index_base=1, **kw):
    """Plan over rows [r0, r1) only (columns: every element).  ``pairs`` uses index_base for
    its column ids, like Plan.create."""
    from .api import Plan

    N = np.asarray(idx1d).shape[0]
    if pairs is not None:
        pairs = (pairs[0], np.asarray(pairs[1]) - index_base)
    rp, cl = row_pairs(N, rows, pairs)
    return Plan.create(term_mats, idx1d, deg, pairs=(rp, cl + index_base), index_base=index_base, **kw)


class ShardedApply:
    """y_local = (A f)[rows of this rank] from f_local = f[rows of this rank].

    plan: a plan over this rank's rows (row_plan), or any object with apply(f) -> y on the
    ranks' tensors; ranges: the row ranges of every rank (partition_rows); block: values per
    element (deg^d); group: the torch.distributed process group (None = default)."""

    def __init__(self, plan, ranges, block, group=None):
        import torch.distributed as dist

        self.plan = plan
        self.ranges = list(ranges)
        self.block = int(block)
        self.group = group
        self.rank = dist.get_rank(group)
        self.world = dist.get_world_size(group)
        if len(self.ranges) != self.world:
            raise ValueError("ShardedApply: %d ranges for %d ranks" % (len(self.ranges), self.world))
        self.counts = [(r1 - r0) * self.block for r0, r1 in self.ranges]

    def gather_f(self, f_local):
        """The all-gather of f (uneven shards are padded to the largest and trimmed)."""
        import torch
        import torch.distributed as dist

        mx = max(self.counts)
        buf = torch.zeros(mx, dtype=f_local.dtype, device=f_local.device)
        buf[:f_local.numel()] = f_local
        parts = [torch.empty_like(buf) for _ in range(self.world)]
        dist.all_gather(parts, buf, group=self.group)
        return torch.cat([p[:c] for p, c in zip(parts, self.counts)])

    def apply(self, f_local):
        r0, r1 = self.ranges[self.rank]
        if f_local.numel() != (r1 - r0) * self.block:
            raise ValueError("ShardedApply: rank %d holds %d values, expected %d"
                             % (self.rank, f_local.numel(), (r1 - r0) * self.block))
        f = self.gather_f(f_local)
        y = self.plan.apply(f)
        return y[r0 * self.block:r1 * self.block]
