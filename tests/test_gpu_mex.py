"""The MEX gateways driven through mexFunction (stand-in mex.h, tests/mexharness.py) on the GPU:
apply_A_mex against the oracle's apply_A loop (apply_A.m:102-236), all pairs and connectivity
pairs; apply_A_T_mex's adjoint and operator gradients against the oracle; the plan cache
rebuilds when an operator is modified in place at the same address."""
import numpy as np
import pytest

import mexharness as M
from cases import problem, rel2
from oracle import asgard_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gw():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return {name: M.Gateway(name) for name in ("apply_A_mex", "apply_A_T_mex")}


def _csr(conn):
    rp = np.zeros(len(conn) + 1)
    rp[1:] = np.cumsum([len(c) for c in conn])
    return rp, np.concatenate([np.asarray(c, dtype=np.float64) for c in conn])


def test_apply_A_mex_matches_oracle(gw):
    import asgkron

    pde, table, idx, mats = problem("continuity2", 4, 2)
    f = np.random.default_rng(0).standard_normal(idx.shape[0] * 4)
    idxd = idx.astype(np.float64)
    want = O.apply_A_loop(mats, idx.astype(np.int64), 2, f)
    (got,) = gw["apply_A_mex"].call(1, mats, idxd, 2, f)
    assert got.shape == (f.size, 1) and rel2(got.ravel(), want) <= 1e-12
    rp, cols = asgkron.connect_nD(table, 4, 4)
    conn = asgkron.connectivity_cells(rp, cols)
    want_c = O.apply_A_loop(mats, idx.astype(np.int64), 2, f, conn=conn)
    rpd, cld = _csr(conn)
    (got_c,) = gw["apply_A_mex"].call(1, mats, idxd, 2, f, rpd, cld)
    assert rel2(got_c.ravel(), want_c) <= 1e-12
    with pytest.raises(M.MexError, match="N\\*deg\\^d"):
        gw["apply_A_mex"].call(1, mats, idxd, 2, f[:-1])


def test_plan_cache_sees_in_place_edits(gw):
    g = gw["apply_A_mex"]
    pde, table, idx, mats = problem("continuity2", 3, 2)
    f = np.random.default_rng(1).standard_normal(idx.shape[0] * 4)
    idxd = g.keep(idx.astype(np.float64))
    ops = g.keep(mats)
    (y1,) = g.call(1, ops, idxd, 2, f)
    (y2,) = g.call(1, ops, idxd, 2, f)  # cached plan
    assert np.array_equal(y1, y2)
    # modify ops{2,1} in place (same mxArray, same data pointer): the digest must change
    cell = M.Mx(g.L.stub_get_cell(ops.ptr, 1))  # (t=1, k=0) of a T x d cell, column-major
    data = g.data(cell)
    data *= 2.0
    mats2 = [[m.copy() for m in row] for row in mats]
    mats2[1][0] = mats2[1][0] * 2.0
    want = O.apply_A_loop(mats2, idx.astype(np.int64), 2, f)
    (y3,) = g.call(1, ops, idxd, 2, f)
    assert rel2(y3.ravel(), want) <= 1e-12 and not np.allclose(y3, y1)
    g.free(ops)
    g.free(idxd)
    g.clear()
    assert not g.L.stub_locked()


def test_apply_A_T_mex_adjoint_and_gradients(gw):
    pde, table, idx, mats = problem("continuity2", 3, 2)
    N = idx.shape[0]
    rng = np.random.default_rng(2)
    f, r = rng.standard_normal(N * 4), rng.standard_normal(N * 4)
    _, A = O.apply_A_loop(mats, idx.astype(np.int64), 2, f, build_A=True)
    fbar, G = gw["apply_A_T_mex"].call(2, mats, idx.astype(np.float64), 2, f, r)
    assert rel2(fbar.ravel(), A.T @ r) <= 1e-12
    want = O.grad_ops_loop(mats, idx.astype(np.int64), 2, f, r)
    T, D = len(mats), len(mats[0])
    applied = 0
    for t in range(T):
        for d in range(D):
            if G[t][d].size == 0:  # identity factor: not differentiated
                continue
            applied += 1
            assert G[t][d].shape == mats[t][d].shape
            assert rel2(G[t][d], want[t][d]) <= 1e-12, (t, d)
    assert applied == T  # continuity2: one applied factor per term
    (fbar1,) = gw["apply_A_T_mex"].call(1, mats, idx.astype(np.float64), 2, f, r)
    assert np.array_equal(fbar1, fbar)
