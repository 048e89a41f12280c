"""Row-sharded apply over ranks: partitioning, per-rank pair lists and the f all-gather,
exercised with world_size 2 over gloo on CPU.  The per-rank compute is the oracle restricted
to the rank's rows (stand-in for the GPU plan, which needs a device)."""
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_partition_rows_balances_prefix_sums():
    from asgkron.shard import partition_rows

    cost = np.array([5, 1, 1, 1, 1, 1, 10, 1, 1, 1, 1, 1])
    parts = partition_rows(cost, 3)
    assert parts[0][0] == 0 and parts[-1][1] == cost.size
    assert all(a[1] == b[0] for a, b in zip(parts, parts[1:]))
    loads = [cost[r0:r1].sum() for r0, r1 in parts]
    assert sum(loads) == cost.sum() and max(loads) <= 13
    assert partition_rows(np.ones(7), 1) == [(0, 7)]
    p = partition_rows(np.ones(3), 5)  # more ranks than rows: some ranges are empty
    assert p[0][0] == 0 and p[-1][1] == 3 and all(r0 <= r1 for r0, r1 in p)


def structured_halo(mats, idx, rows, drop_tol=1e-13):
    """The halo of rows [r0, r1) as the structure analysis defines it, restated in numpy: the
    columns j outside the range such that some term's identity dimensions match row i's 1-D
    indices and every applied factor's deg x deg block (i, j) is nonzero (0-based, ascending).
    idx is 1-based [N, d]."""
    T, D = len(mats), len(mats[0])
    N = idx.shape[0]
    deg = mats[0][0].shape[0] // int(idx.max())
    ident, zero = [[None] * D for _ in range(T)], [[None] * D for _ in range(T)]
    for t in range(T):
        for m in range(D):
            A = np.asarray(mats[t][m])
            thr = drop_tol * np.abs(A).max()
            ident[t][m] = bool(np.all(np.abs(A - np.eye(A.shape[0])) <= thr))
            nb = A.shape[0] // deg
            zero[t][m] = np.abs(A.reshape(nb, deg, nb, deg)).max(axis=(1, 3)) <= thr
    r0, r1 = rows
    need = set()
    for i in range(r0, r1):
        for j in range(N):
            if r0 <= j < r1:
                continue
            for t in range(T):
                ok = True
                for m in range(D):
                    a, b = idx[i, m] - 1, idx[j, m] - 1
                    if ident[t][m]:
                        ok = a == b
                    else:
                        ok = not zero[t][m][a, b]
                    if not ok:
                        break
                if ok:
                    need.add(j)
                    break
    return np.array(sorted(need), dtype=np.int64)


def test_exchange_lists_route_every_halo_block():
    from asgkron.shard import exchange_lists

    ranges = [(0, 3), (3, 5), (5, 9)]
    halos = [[3, 4, 7], [0, 8], [2, 4]]
    s0, r0 = exchange_lists(ranges, halos, 0)
    assert [list(x) for x in s0] == [[], [0], [2]] and r0 == [0, 2, 1]
    s1, r1 = exchange_lists(ranges, halos, 1)
    assert [list(x) for x in s1] == [[0, 1], [], [1]] and r1 == [1, 0, 1]
    s2, r2 = exchange_lists(ranges, halos, 2)
    assert [list(x) for x in s2] == [[2], [3], []] and r2 == [1, 1, 0]
    with pytest.raises(ValueError):
        exchange_lists([(0, 3), (3, 5)], [[7], []], 0)  # element 7 lies in no range


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out_path):
    sys.path[:0] = [ROOT, os.path.join(ROOT, "dg-sparsegrid_gb300"), os.path.join(ROOT, "tests")]
    import torch
    import torch.distributed as dist

    from cases import problem
    from oracle import asgard_oracle as O
    from asgkron.shard import ShardedApply, partition_rows
    from test_shard_cpu import structured_halo

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        _, _, idx, mats = problem("continuity2", 4, 2)
        deg = 2
        N, D = idx.shape
        B = deg ** D
        idx64 = idx.astype(np.int64)
        f = np.random.default_rng(0).standard_normal(N * B)
        ranges = partition_rows(np.full(N, N), world)
        r0, r1 = ranges[rank]
        halo = structured_halo(mats, idx, (r0, r1))

        class OracleSlice:  # the rank's row-slice plan: f = rows + halo, y = rows
            def apply(self, fc):
                full = np.zeros(N * B)
                elems = np.concatenate([np.arange(r0, r1), halo]).astype(np.int64)
                full.reshape(N, B)[elems] = fc.numpy().reshape(-1, B)
                if r1 == r0:
                    return torch.zeros(0, dtype=torch.float64)
                return torch.from_numpy(O.apply_A_rows(mats, idx64, deg, full, rows=np.arange(r0, r1)))

        sharded = ShardedApply(OracleSlice(), ranges, B, halo=halo)
        f_local = torch.from_numpy(f.reshape(N, B)[r0:r1].ravel().copy())
        # the exchanged input is the rank's rows followed by exactly its halo blocks
        got = sharded.gather_f(f_local).clone()
        want_in = np.concatenate([f.reshape(N, B)[r0:r1], f.reshape(N, B)[halo]]).ravel()
        in_ok = bool(np.array_equal(got.numpy(), want_in))
        y_local = sharded.apply(f_local)
        y_again = sharded.apply(f_local)  # buffers reused: same result
        counts = [(b - a) * B for a, b in ranges]
        parts = [torch.zeros(max(counts), dtype=torch.float64) for _ in range(world)]
        buf = torch.zeros(max(counts), dtype=torch.float64)
        buf[:y_local.numel()] = y_local
        dist.all_gather(parts, buf)
        flags = [None] * world
        dist.all_gather_object(flags, (in_ok, bool(torch.equal(y_local, y_again)), int(halo.size)))
        if rank == 0:
            y = torch.cat([p[:c] for p, c in zip(parts, counts)]).numpy()
            want = O.apply_A_rows(mats, idx64, deg, f)
            err = np.linalg.norm(y - want) / np.linalg.norm(want)
            with open(out_path, "w") as fh:
                fh.write("%.17g %r %r" % (float(err), flags, [[int(a), int(b)] for a, b in ranges]))
    finally:
        dist.destroy_process_group()


def test_sharded_apply_two_gloo_ranks(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    import ast

    out = str(tmp_path / "res.txt")
    mp.start_processes(_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    err, rest = open(out).read().split(" ", 1)
    flags = ast.literal_eval(rest[:rest.index("]") + 1])
    assert float(err) <= 1e-14, (err, rest)
    assert all(a and b for a, b, _ in flags), flags
    # each rank receives only its halo: far less than the other rank's whole share
    assert all(0 < h < 100 for _, _, h in flags), flags


def test_partition_problems_covers_and_balances():
    from asgkron.batch import partition_problems

    rng = np.random.default_rng(7)
    for count in (0, 1, 5, 64, 256):
        costs = rng.lognormal(0.0, 2.0, count)
        for nparts in (1, 2, 3, 8):
            parts = partition_problems(costs, nparts)
            assert len(parts) == nparts
            flat = sorted(k for p in parts for k in p)
            assert flat == list(range(count))  # each problem on exactly one rank
            assert all(p == sorted(p) for p in parts)
            if count:
                loads = [sum(costs[k] for k in p) for p in parts]
                assert max(loads) <= sum(costs) / nparts + max(costs) + 1e-9
            assert parts == partition_problems(list(costs), nparts)  # deterministic
    assert partition_problems([5.0, 1.0, 1.0, 1.0, 1.0, 1.0], 2) == [[0], [1, 2, 3, 4, 5]]
    with pytest.raises(ValueError):
        partition_problems([1.0], 0)
    with pytest.raises(ValueError):
        partition_problems([-1.0], 2)


def test_batch_draws_follow_the_generator():
    """bench.batch_draws advances the random stream as the batched workload draws its problems:
    (d, lev, deg) of every problem equal an explicit replay of the draw order (scalars, d^2
    operators, f), and N is the element count of the problem's table."""
    import asgkron
    import bench

    draws = bench.batch_draws(6, 4)
    rng = np.random.default_rng(3)
    for d, lev, deg, N in draws:
        assert (d, lev, deg) == (int(rng.choice([2, 3, 4])), int(rng.integers(3, 5)), int(rng.integers(2, 5)))
        assert N == asgkron.hash_table_sparse_nD([lev] * d, 8).idx1d().shape[0]
        n = deg * 2 ** lev
        [rng.normal(0.0, 1.0 / np.sqrt(deg), (n, n)) for _ in range(d * d)]
        rng.standard_normal(N * deg ** d)
    assert bench.batch_draws(3, 4) == draws[:3]


def _batch_worker(rank, world, port, out_path):
    import torch.distributed as dist

    sys.path[:0] = [ROOT, os.path.join(ROOT, "dg-sparsegrid_gb300")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from asgkron.batch import partition_problems

        draws = bench.batch_draws(24, 4)
        costs = bench.batch_costs(draws)
        mine = partition_problems(costs, world)[rank]
        got = [None] * world
        dist.all_gather_object(got, (mine, draws))
        if rank == 0:
            with open(out_path, "w") as fh:
                fh.write(repr((got, costs)))
    finally:
        dist.destroy_process_group()


def test_batched_problem_shards_two_gloo_ranks(tmp_path):
    """Two ranks draw the same problems and take disjoint, covering, cost-balanced shares of
    them without exchanging any problem data (the batched configuration's sharding)."""
    pytest.importorskip("torch")
    import torch.multiprocessing as mp

    out = str(tmp_path / "shards.txt")
    mp.start_processes(_batch_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    import ast

    got, costs = ast.literal_eval(open(out).read())
    (m0, d0), (m1, d1) = got
    assert d0 == d1
    assert sorted(m0 + m1) == list(range(24)) and not set(m0) & set(m1)
    l0, l1 = sum(costs[k] for k in m0), sum(costs[k] for k in m1)
    assert max(l0, l1) <= sum(costs) / 2 + max(costs)
