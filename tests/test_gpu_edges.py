"""Edge cases of the apply path: one dimension and degree one, the largest element blocks,
operators with no non-zero block, empty and ragged pair lists, an empty element table,
non-finite operators, aliasing buffers."""
import numpy as np
import pytest

from cases import problem, random_problem, rel2
from oracle import asgard_oracle as O

torch = pytest.importorskip("torch")
FP64_TOL = 1e-12
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def _t(x, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(x)).to(dev, dtype)


@pytest.mark.parametrize("d,lev,deg", [(1, 3, 1), (1, 6, 2), (2, 2, 1), (4, 1, 8), (3, 1, 8)])
def test_extreme_shapes_vs_oracle(dev, d, lev, deg):
    """deg 1 (1-value blocks), one dimension, and the largest blocks (8^4 = 4096, 8^3 = 512)."""
    import asgkron

    table, idx, mats = random_problem(70 + d * 10 + deg, d, lev, deg)
    N = idx.shape[0]
    f = np.random.default_rng(d + deg).standard_normal(N * deg ** d)
    for structure in ("none", "detect"):
        plan = asgkron.Plan.create(mats, idx, deg, structure=structure)
        y = plan.apply(_t(f, dev))
        torch.cuda.synchronize()
        want = O.apply_A_loop(mats, idx.astype(np.int64), deg, f)
        assert rel2(y.cpu().numpy(), want) <= FP64_TOL, structure
        y32 = plan.apply(_t(f, dev, torch.float32))
        torch.cuda.synchronize()
        assert rel2(y32.double().cpu().numpy(), want) <= 1e-6, structure


def test_zero_operators_and_empty_rows(dev):
    """Operators with no non-zero block leave no work entries: y is zero (written, not left
    as it was).  Rows with an empty pair list are zero as well."""
    import asgkron

    pde, table, idx, mats = problem("continuity2", 3, 2)
    N = idx.shape[0]
    zero = [[np.zeros_like(m) for m in row] for row in mats]
    plan = asgkron.Plan.create(zero, idx, 2)
    assert plan.stats()["num_entries"] == 0
    y = torch.full((N * 4,), 7.0, dtype=torch.float64, device=dev)
    plan.apply(_t(np.ones(N * 4), dev), y)
    torch.cuda.synchronize()
    assert float(y.abs().max()) == 0.0
    # ragged list with empty rows 0 and 2
    lens = np.array([0 if i in (0, 2) else (i % 5) + 1 for i in range(N)])
    rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
    rng = np.random.default_rng(3)
    cols = np.concatenate([np.sort(rng.choice(N, size=k, replace=False)) for k in lens]).astype(np.int32)
    f = rng.standard_normal(N * 4)
    conn = [list(cols[rp[i]:rp[i + 1]] + 1) for i in range(N)]
    want = O.apply_A_loop(mats, idx.astype(np.int64), 2, f, conn=conn)
    for structure in ("none", "detect"):
        p = asgkron.Plan.create(mats, idx, 2, pairs=(rp, cols + 1), structure=structure)
        got = p.apply(_t(f, dev))
        torch.cuda.synchronize()
        got = got.cpu().numpy()
        assert not np.any(got.reshape(N, 4)[[0, 2]])
        assert rel2(got, want) <= FP64_TOL, structure


def test_empty_element_table(dev):
    import asgkron

    mats = [[np.eye(4)]]
    plan = asgkron.Plan.create(mats, np.zeros((0, 1), dtype=np.int32), 2)
    st = plan.stats()
    assert st["dof"] == 0 and st["num_entries"] == 0


def test_rejected_inputs(dev):
    import ctypes as C

    import asgkron
    from asgkron._lib import AsgError, check

    pde, table, idx, mats = problem("continuity2", 3, 2)
    bad = [[m.copy() for m in row] for row in mats]
    bad[1][0][3, 5] = np.nan
    with pytest.raises(AsgError, match="non-finite"):
        asgkron.Plan.create(bad, idx, 2)
    plan = asgkron.Plan.create(mats, idx, 2)
    f = torch.zeros(plan.dof, dtype=torch.float64, device=dev)
    with pytest.raises(AsgError, match="alias"):
        check(asgkron.lib().asg_apply_f64(plan.handle, C.c_void_p(f.data_ptr()), C.c_void_p(f.data_ptr()), None))
    with pytest.raises(AsgError, match="unknown kernel kind"):
        plan.set_kernel(9)
    with pytest.raises(AsgError):
        plan.set_kernel(asgkron._lib.KERNEL_SINGLE_TMA)  # deg 2: the TMA kernels need deg 4, d 6
