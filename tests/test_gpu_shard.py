"""Row-slice plans of the row-sharded apply, on one GPU: each rank's plan takes its rows'
blocks followed by its halo (the exchange emulated by indexing f) and writes its rows only;
together they reproduce the full plan's y bitwise (same entries, same order, same kernel).
The halo the C++ structure analysis finds equals the numpy restatement used on CPU ranks."""
import numpy as np
import pytest

from cases import problem
from test_shard_cpu import structured_halo

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,lev,deg,conn,nranks", [("continuity2", 4, 2, False, 2), ("continuity2", 4, 2, True, 3),
                                                      ("continuity6", 3, 4, False, 4), ("diffusion2", 5, 4, True, 2)])
def test_row_slices_reassemble_full_apply(name, lev, deg, conn, nranks):
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
        halo = p.halo() - 1
        if pairs is None:
            assert np.array_equal(halo, structured_halo(mats, idx, (r0, r1))), (r0, r1)
        assert np.all((halo < r0) | (halo >= r1)) and np.all(np.diff(halo) > 0)
        assert p.dof == (r1 - r0) * B and p.dof_in == (r1 - r0 + halo.size) * B
        assert p.stats()["kernel_kind"] == full.stats()["kernel_kind"]
        elems = torch.from_numpy(np.concatenate([np.arange(r0, r1), halo])).cuda()
        fc = f.view(N, B).index_select(0, elems).reshape(-1).contiguous()
        parts.append(p.apply(fc))
        # host pointers: the same slice through asg_apply_host_f64
        yh = p.apply_host(fc.cpu().numpy())
        assert np.array_equal(yh, parts[-1].cpu().numpy())
    torch.cuda.synchronize()
    assert torch.equal(torch.cat(parts), y)


def test_row_slice_halo_is_smaller_than_an_all_gather():
    """continuity6 SG 4, deg 4 in four slices: the four halos hold 734 blocks where an all-gather
    of f would move 1,503 (the finest elements come first in the table and read few others; the
    coarsest slice reads nearly every other element)."""
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from asgkron.shard import partition_rows, row_plan

    _, _, idx, mats = problem("continuity6", 4, 4)
    N = idx.shape[0]
    halo, gather = [], []
    for r0, r1 in partition_rows(np.full(N, 1), 4):
        p = row_plan(mats, idx, 4, (r0, r1))
        halo.append(p.halo().size)
        gather.append(N - (r1 - r0))
        p.close()
    assert halo == [64, 113, 195, 362] and sum(gather) == 1503, (halo, gather)


def test_row_slice_rejects_what_it_does_not_run():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from asgkron._lib import ASG_ERR_UNSUPPORTED, ASG_ERR_INVALID, AsgError
    import asgkron
    from asgkron.shard import row_plan

    _, _, idx, mats = problem("continuity2", 3, 2)
    N = idx.shape[0]
    p = row_plan(mats, idx, 2, (1, N // 2))
    yb = torch.zeros(p.dof, dtype=torch.float64, device="cuda")
    with pytest.raises(AsgError) as e:
        p.apply_T(yb, torch.zeros(p.dof_in, dtype=torch.float64, device="cuda"))
    assert e.value.status == ASG_ERR_UNSUPPORTED
    with pytest.raises(AsgError) as e:
        p.update_elements(idx)
    assert e.value.status == ASG_ERR_UNSUPPORTED
    with pytest.raises(AsgError) as e:
        asgkron.Plan.create(mats, idx, 2, rows=(3, 2))
    assert e.value.status == ASG_ERR_INVALID
    with pytest.raises(ValueError):
        p.apply(torch.zeros(p.dof, dtype=torch.float64, device="cuda"))  # f must hold rows + halo
    # an empty slice writes nothing and needs nothing
    q = row_plan(mats, idx, 2, (2, 2))
    assert q.dof == 0 and q.halo().size == 0
