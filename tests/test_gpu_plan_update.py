"""The element-table update of a plan (asg_plan_update_elements) against fresh plans, the
oracle, and the reference's adaptive gold run driven by GPU RK3 steps."""
import os

import numpy as np
import pytest

from cases import rel2

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _need_gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.parametrize("structure", ["detect", "none"])
def test_update_elements_equals_a_fresh_plan(structure):
    """Coarsen and refine a continuity2 table, then update the plan in place: the apply, the
    adjoint and the operator gradients equal a plan created on the new table, bitwise; y equals
    the oracle's loop."""
    _need_gpu()
    import asgkron
    from asgkron import pdes
    from asgkron.adapt import adapt, operator_extent
    from oracle import asgard_oracle as O

    pde = pdes.continuity2(3)
    deg, max_lev = 2, 5
    table = asgkron.hash_table_sparse_nD(pde.levels, max_lev)
    mats = pde.term_mats(deg, construction_level=max_lev)
    plan = asgkron.Plan.create(mats, table.idx1d(), deg, structure=structure, op_blocks=operator_extent(mats, deg))
    f = np.random.default_rng(11).standard_normal(plan.dof) * np.repeat(np.linspace(1.0, 0.01, table.num_elems), 4)
    res = adapt(table, f, deg, max_lev, 0.6)
    assert res.added > 0 and res.removed.size > 0
    plan.update_elements(res.table.idx1d())
    fresh = asgkron.Plan.create(mats, res.table.idx1d(), deg, structure=structure)
    assert plan.stats()["num_entries"] == fresh.stats()["num_entries"]
    fv = torch.from_numpy(res.fval).cuda()
    y, y0 = plan.apply(fv), fresh.apply(fv)
    assert torch.equal(y, y0)
    r = torch.from_numpy(np.random.default_rng(12).standard_normal(plan.dof)).cuda()
    assert torch.equal(plan.apply_T(r), fresh.apply_T(r))
    g, g0 = plan.grad_ops(fv, r), fresh.grad_ops(fv, r)
    for a, b in zip(sum(g, []), sum(g0, [])):
        assert (a is None and b is None) or torch.equal(a, b)
    want = O.apply_A_loop(mats, res.table.idx1d().astype(np.int64), deg, res.fval)
    assert rel2(y.cpu().numpy(), want) <= 1e-12
    # a second update back to the first table (a shrink) and FP32
    plan.update_elements(table.idx1d())
    f32 = torch.from_numpy(f).cuda().float()
    y1 = plan.apply(f32)
    p1 = asgkron.Plan.create(mats, table.idx1d(), deg, structure=structure)
    assert torch.equal(y1, p1.apply(f32))


def test_update_elements_with_pair_lists_and_base0():
    """A connectivity-list plan (0-based indices) takes a new table with its own connect_nD
    pairs in place: equal to a fresh plan on that table and pair list, bitwise, both work
    models."""
    _need_gpu()
    import asgkron
    from asgkron import pdes

    pde = pdes.continuity2(3)
    deg = 2
    mats = pde.term_mats(deg, construction_level=5)
    t1 = asgkron.hash_table_sparse_nD([3, 3], 5)
    t2 = asgkron.hash_table_sparse_nD([4, 4], 5)
    for structure in ("detect", "none"):
        rp1, cl1 = asgkron.connect_nD(t1, 3, 3)
        rp2, cl2 = asgkron.connect_nD(t2, 4, 4)
        plan = asgkron.Plan.create(mats, t1.idx1d() - 1, deg, pairs=(rp1, cl1), index_base=0,
                                   structure=structure, op_blocks=[32, 32])
        plan.update_elements(t2.idx1d() - 1, (rp2, cl2))
        fresh = asgkron.Plan.create(mats, t2.idx1d() - 1, deg, pairs=(rp2, cl2), index_base=0, structure=structure)
        assert plan.stats()["num_pairs"] == fresh.stats()["num_pairs"] == rp2[-1]
        f = torch.from_numpy(np.random.default_rng(5).standard_normal(fresh.dof)).cuda()
        assert torch.equal(plan.apply(f), fresh.apply(f))
        assert torch.equal(plan.apply(f.float()), fresh.apply(f.float()))


def test_update_elements_capacity_and_argument_errors():
    _need_gpu()
    import asgkron
    from asgkron import pdes
    from asgkron._lib import ASG_ERR_CAPACITY, ASG_ERR_INVALID, AsgError

    pde = pdes.continuity2(2)
    deg = 2
    small = asgkron.hash_table_sparse_nD([2, 2], 5)
    big = asgkron.hash_table_sparse_nD([4, 4], 5)
    mats = pde.term_mats(deg, construction_level=5)
    plan = asgkron.Plan.create(mats, small.idx1d(), deg)  # packs only what level 2 reaches
    f = torch.from_numpy(np.random.default_rng(3).standard_normal(plan.dof)).cuda()
    y0 = plan.apply(f).clone()
    with pytest.raises(AsgError) as e:
        plan.update_elements(big.idx1d())
    assert e.value.status == ASG_ERR_CAPACITY
    bad = small.idx1d().copy()
    bad[0, 0] = 0  # below the 1-based index
    with pytest.raises(AsgError) as e:
        plan.update_elements(bad)
    assert e.value.status == ASG_ERR_INVALID
    with pytest.raises(AsgError) as e:  # a pair list whose column lies outside the table
        plan.update_elements(small.idx1d(), (np.array([0] + [1] * small.num_elems), np.array([small.num_elems + 1])))
    assert e.value.status == ASG_ERR_INVALID
    assert torch.equal(plan.apply(f), y0)  # errors left the plan as it was
    # reserving the operators' extent admits the finer table
    from asgkron.adapt import update_plan
    p2 = update_plan(plan, big)
    assert p2 is not plan
    p3 = update_plan(p2, small)
    assert p3 is p2 and torch.equal(p3.apply(f), y0)


def test_adaptive_continuity2_gold_run_with_gpu_steps_and_plan_updates():
    """The reference's adaptive run continuity2_ad_sg_l3_d4 (RK3, five steps, 20 -> 112
    elements) with every step on the GPU (FP64 RK3 on the run's table), the plan kept across
    tables by update_plan: the states match the gold files."""
    _need_gpu()
    import asgkron
    from asgkron import pdes
    from asgkron.adapt import AdaptiveRun, operator_extent, update_plan
    from asgkron.steppers import RK3Stepper

    ta = np.load(os.path.join(G, "time_advance.npz"))
    pde = pdes.continuity2(3, 0.0)
    run = AdaptiveRun(pde, 4, asgkron.hash_table_sparse_nD([3, 3], 8), 1e-3)
    dt = pdes.continuity2(3, 0.0).dt(0.01)
    state = {"plan": None, "updates": 0, "rebuilds": 0}

    def step(r, fv, t):
        if state["plan"] is None:
            # operators at the maximum level (single partial terms: every table's operators are
            # their leading blocks), their whole extent reserved
            top = r.pde.rechain_term_mats(4, [8, 8], 8, r._pterms)
            state["plan"] = asgkron.Plan.create(top, r.idx1d, 4, op_blocks=operator_extent(top, 4))
            state["rebuilds"] += 1
        else:
            new = update_plan(state["plan"], r.table, term_mats=r.term_mats())
            state["updates" if new is state["plan"] else "rebuilds"] += 1
            state["plan"] = new
        x = torch.from_numpy(np.ascontiguousarray(fv)).cuda()
        RK3Stepper(state["plan"], pde, r.idx1d).step(x, t, dt)
        return x.cpu().numpy()

    f = run.initial()
    for i in range(5):
        f = run.advance(f, i * dt, step)
        g = ta["continuity2_ad_sg_l3_d4_t%d" % i]
        assert f.size == g.size, (i, f.size, g.size)
        assert np.linalg.norm(f - g) <= 1e-13 * np.linalg.norm(g), i
    assert run.table.num_elems == 112
    assert state["updates"] > 0 and state["rebuilds"] == 1, state
