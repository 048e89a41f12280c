"""Per-rank plans of the row-sharded apply, on one GPU: the plans over each rank's rows
together reproduce the full plan's y bitwise (same entries, same order, same kernel)."""
import numpy as np
import pytest

from cases import problem

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,lev,deg,conn,nranks", [("continuity2", 4, 2, False, 2), ("continuity2", 4, 2, True, 3),
                                                      ("continuity6", 3, 4, False, 4), ("diffusion2", 5, 4, True, 2)])
def test_row_plans_reassemble_full_apply(name, lev, deg, conn, nranks):
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import asgkron
    from asgkron.shard import partition_rows, row_plan

    pde, table, idx, mats = problem(name, lev, deg)
    N, D = idx.shape
    B = deg ** D
    pairs = None
    if conn:
        rp, cl = asgkron.connect_nD(table, max(pde.levels), max(pde.levels))
        pairs = (rp, cl + 1)
    full = asgkron.Plan.create(mats, idx, deg, pairs=pairs)
    f = torch.from_numpy(np.random.default_rng(9).standard_normal(N * B)).cuda()
    y = full.apply(f)
    cost = np.full(N, N) if pairs is None else np.diff(pairs[0])
    ranges = partition_rows(cost, nranks)
    parts = []
    for r0, r1 in ranges:
        p = row_plan(mats, idx, deg, (r0, r1), pairs=pairs)
        assert p.stats()["kernel_kind"] == full.stats()["kernel_kind"]
        parts.append(p.apply(f)[r0 * B:r1 * B])
    torch.cuda.synchronize()
    assert torch.equal(torch.cat(parts), y)
