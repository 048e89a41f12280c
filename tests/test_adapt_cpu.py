"""Adaptive element tables (adapt.m, get_child_elements.m) on CPU, and the rebuilt plan on
the GPU against the oracle."""
import numpy as np
import pytest

from cases import rel2


def test_child_elements_methods():
    from asgkron.adapt import child_elements

    # 2-D element (lev 1, 0), pos (0, 0): dimension 1 has two daughters (lev >= 1), dimension 2 one
    c1 = child_elements((1, 0), (0, 0), 4, method=1)
    assert c1 == [((2, 0), (0, 0)), ((2, 0), (1, 0)), ((1, 1), (0, 0))]
    c2 = child_elements((1, 0), (0, 0), 4, method=2)
    assert c2[:3] == c1 and sorted(c2[3:]) == [((2, 1), (0, 0)), ((2, 1), (1, 0))]
    # at lev = max_lev - 1 there is nothing to add
    assert child_elements((3, 3), (5, 1), 4) == []
    assert child_elements((0,), (0,), 1) == []


def test_adapt_coarsen_and_refine_rules():
    import asgkron
    from asgkron.adapt import NEW_ELEMENT_VALUE, adapt, child_elements, md_keys

    table = asgkron.hash_table_sparse_nD([2, 2], 4)
    N, d, deg = table.num_elems, 2, 2
    B = deg ** d
    f = np.full((N, B), 0.06)
    f[0] = 1.0           # refined: max |f|
    f[3, 1] = -0.7       # refined (>= 0.5 = rel * max)
    f[5] = 1e-3          # coarsened (<= 0.05 = 0.1 * rel * max)
    res = adapt(table, f.ravel(), deg, 4, 0.5)
    assert list(res.removed) == [5]
    kept = [i for i in range(N) if i != 5]
    nk = len(kept)
    assert np.array_equal(res.table.levels[:nk], table.levels[kept])
    assert np.array_equal(res.table.cells[:nk], table.cells[kept])
    assert np.array_equal(res.fval.reshape(-1, B)[:nk], f[kept])
    # appended: the daughters of elements 0 and 3 not yet present, in discovery order
    present = {(tuple(l), tuple(c)) for l, c in zip(table.levels[kept].tolist(), table.cells[kept].tolist())}
    want = []
    for e in (0, 3):
        for ch in child_elements(table.levels[e], table.cells[e], 4):
            if ch not in present and ch not in want:
                want.append(ch)
    got = [(tuple(l), tuple(c)) for l, c in zip(res.table.levels[nk:].tolist(), res.table.cells[nk:].tolist())]
    assert got == want and res.added == len(want) > 0
    assert np.all(res.fval.reshape(-1, B)[nk:] == NEW_ELEMENT_VALUE)
    # keys follow md_lev_pos_to_idx and are unique
    assert np.array_equal(md_keys(table.levels, table.cells, 4), table.keys)
    assert len(set(res.table.keys.tolist())) == res.table.num_elems
    # zero field: nothing happens
    z = adapt(table, np.zeros(N * B), deg, 4, 0.5)
    assert z.table.num_elems == N and z.added == 0 and z.removed.size == 0


@pytest.mark.gpu
@pytest.mark.gpu
def test_rebuilt_plan_matches_oracle_after_adapt():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import asgkron
    from asgkron import pdes
    from asgkron.adapt import adapt, rebuild_plan
    from oracle import asgard_oracle as O

    pde = pdes.continuity2(3)
    deg, max_lev = 2, 5
    table = asgkron.hash_table_sparse_nD(pde.levels, max_lev)
    mats = pde.term_mats(deg, construction_level=max_lev)  # rows for every level up to max_lev
    plan = asgkron.Plan.create(mats, table.idx1d(), deg)
    f = np.random.default_rng(11).standard_normal(plan.dof) * np.repeat(np.linspace(1.0, 0.01, table.num_elems), 4)
    res = adapt(table, f, deg, max_lev, 0.6)
    assert res.added > 0 and res.removed.size > 0
    p2 = rebuild_plan(plan, res.table)
    y = p2.apply(torch.from_numpy(res.fval).cuda())
    torch.cuda.synchronize()
    want = O.apply_A_loop(mats, res.table.idx1d().astype(np.int64), deg, res.fval)
    assert rel2(y.cpu().numpy(), want) <= 1e-12
