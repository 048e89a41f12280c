"""Adjoint (A^T ybar) and operator gradients on the GPU, and the torch.autograd harness.

References: the oracle's explicit krond differentiation (small cases), FP64 central finite
differences (step 1e-6) and the inner-product identity <A f, r> = <f, A^T r>.
"""
import numpy as np
import pytest

from cases import problem, random_problem, rel2
from oracle import asgard_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def _t(x, dev, dtype=torch.float64):
    return torch.from_numpy(np.ascontiguousarray(x)).to(dev, dtype)


@pytest.mark.parametrize("case", ["continuity2", "random_d2", "random_d3"])
@pytest.mark.parametrize("structure", ["none", "detect"])
def test_adjoint_and_grad_vs_oracle(dev, case, structure):
    import asgkron

    if case == "continuity2":
        _, _, idx, mats = problem("continuity2", 3, 2)
        deg = 2
    elif case == "random_d2":
        _, idx, mats = random_problem(21, 2, 2, 3)
        deg = 3
    else:
        _, idx, mats = random_problem(22, 3, 2, 2)
        deg = 2
    idx64 = idx.astype(np.int64)
    N, D = idx.shape
    n = N * deg ** D
    rng = np.random.default_rng(5)
    f, r = rng.standard_normal(n), rng.standard_normal(n)
    plan = asgkron.Plan.create(mats, idx, deg, structure=structure)
    # adjoint: dense A from the oracle
    _, A = O.apply_A_loop(mats, idx64, deg, f, build_A=True)
    fbar = plan.apply_T(_t(r, dev))
    torch.cuda.synchronize()
    assert rel2(fbar.cpu().numpy(), A.T @ r) <= 1e-12
    # operator gradients
    G = plan.grad_ops(_t(f, dev), _t(r, dev))
    want = O.grad_ops_loop(mats, idx64, deg, f, r)
    active = plan.active_factors()
    for t in range(len(mats)):
        for d in range(D):
            if not active[t][d]:
                assert G[t][d] is None
                continue
            got = G[t][d].cpu().numpy()
            nn = got.shape[0]
            w = want[t][d][:nn, :nn]
            assert np.abs(got - w).max() <= 1e-12 * max(1.0, np.abs(w).max()), (t, d)
    # FP32 variants
    fbar32 = plan.apply_T(_t(r, dev, torch.float32))
    G32 = plan.grad_ops(_t(f, dev, torch.float32), _t(r, dev, torch.float32))
    torch.cuda.synchronize()
    assert rel2(fbar32.double().cpu().numpy(), A.T @ r) <= 1e-6
    for t in range(len(mats)):
        for d in range(D):
            if active[t][d]:
                a, b = G32[t][d].double().cpu().numpy(), G[t][d].cpu().numpy()
                assert np.linalg.norm(a - b) <= 1e-5 * max(1e-30, np.linalg.norm(b))


def _single_factor_grad_numpy(mats, idx0, f, r, deg):
    """dL/dA_t for terms I x .. x A_t x .. x I over all pairs: for identity-compatible pairs
    (i, j), block (I_t(i), J_t(j)) of G_t gains R_i^(t) Z_j^(t)T, the mode-t unfoldings."""
    N, D = idx0.shape
    B = deg ** D
    G = [np.zeros_like(np.asarray(mats[t][t])) for t in range(D)]
    R = r.reshape(N, *([deg] * D))
    F = f.reshape(N, *([deg] * D))
    for t in range(D):
        others = [m for m in range(D) if m != t]
        groups = {}
        for e in range(N):
            groups.setdefault(tuple(idx0[e, others]), []).append(e)
        for i in range(N):
            Ri = np.moveaxis(R[i], t, 0).reshape(deg, -1)
            for j in groups[tuple(idx0[i, others])]:
                Zj = np.moveaxis(F[j], t, 0).reshape(deg, -1)
                a, b = idx0[i, t], idx0[j, t]
                G[t][a * deg:(a + 1) * deg, b * deg:(b + 1) * deg] += Ri @ Zj.T
    return G


@pytest.mark.parametrize("lev", [2, 3])
def test_single_factor_gradients_chunked_kernel(dev, lev):
    """continuity6 deg 4 (one applied factor per term): the chunked gradient kernel, on all
    pairs and on the same pairs given as an explicit list, against the mode-unfolding
    contraction in numpy, FP64 and FP32, and bitwise repeatable."""
    import asgkron

    _, _, idx, mats = problem("continuity6", lev, 4)
    N = idx.shape[0]
    rng = np.random.default_rng(40 + lev)
    f, r = rng.standard_normal(N * 4096), rng.standard_normal(N * 4096)
    plan = asgkron.Plan.create(mats, idx, 4)
    listed = asgkron.Plan.create(mats, idx, 4, pairs=(np.arange(N + 1) * N, np.tile(np.arange(N) + 1, N)))
    want = _single_factor_grad_numpy(mats, idx.astype(np.int64) - 1, f, r, 4)
    G = plan.grad_ops(_t(f, dev), _t(r, dev))
    G2 = plan.grad_ops(_t(f, dev), _t(r, dev))
    Gl = listed.grad_ops(_t(f, dev), _t(r, dev))
    torch.cuda.synchronize()
    for t in range(6):
        got = G[t][t].cpu().numpy()
        assert np.abs(got - want[t]).max() <= 1e-12 * np.abs(want[t]).max(), t
        assert np.abs(Gl[t][t].cpu().numpy() - want[t]).max() <= 1e-12 * np.abs(want[t]).max(), t
        assert torch.equal(G[t][t], G2[t][t])
    G32 = plan.grad_ops(_t(f, dev, torch.float32), _t(r, dev, torch.float32))
    torch.cuda.synchronize()
    for t in range(6):
        a, b = G32[t][t].double().cpu().numpy(), want[t]
        assert np.linalg.norm(a - b) <= 1e-5 * np.linalg.norm(b), t


def test_continuity6_gradients_fd(dev):
    """Differentiation configuration: continuity6 SG lev 4, deg 4, f ~ N(0,1) seed 4,
    y* ~ N(0,1) seed 5, L = 1/2 ||A f - y*||^2.  Gradients with respect to f and to the six 1-D
    coefficient matrices against FP64 central differences (step 1e-6) on 64 random entries."""
    import asgkron

    _, _, idx, mats = problem("continuity6", 4, 4)
    B = 4096
    N = idx.shape[0]
    f = np.random.default_rng(4).standard_normal(N * B)
    ys = np.random.default_rng(5).standard_normal(N * B)
    plan = asgkron.Plan.create(mats, idx, 4)
    ft, yst = _t(f, dev), _t(ys, dev)

    def dloss(yp, ym):
        # L(+) - L(-) summed elementwise: 1/2 (y+ - y-) (y+ + y- - 2 y*); the same central
        # difference without subtracting two ~1e10 sums from each other
        return 0.5 * float(torch.sum((yp - ym) * (yp + ym - 2 * yst)))

    r = plan.apply(ft) - yst
    fbar = plan.apply_T(r)
    G = plan.grad_ops(ft, r)
    torch.cuda.synchronize()
    # <A f, r> = <f, A^T r>
    lhs = float(torch.dot(plan.apply(ft), r))
    rhs = float(torch.dot(ft, fbar))
    assert abs(lhs - rhs) <= 1e-11 * abs(lhs)
    rng = np.random.default_rng(64)
    h = 1e-6
    idxs = rng.choice(N * B, 32, replace=False)
    fb = fbar.cpu().numpy()
    for k in idxs:
        e = torch.zeros_like(ft)
        e[int(k)] = h
        fd = dloss(plan.apply(ft + e), plan.apply(ft - e)) / (2 * h)
        assert abs(fd - fb[k]) <= 1e-6 * max(1.0, abs(fb[k])), (k, fd, fb[k])
    active = plan.active_factors()
    assert sum(map(sum, active)) == 6  # one coefficient matrix per term
    picks = []
    for t in range(6):
        g = G[t][t].cpu().numpy()
        nz = np.argwhere(np.abs(g) > 0)
        for q in rng.choice(len(nz), 5, replace=False):
            picks.append((t, *nz[q]))
    # The gradient is the full derivative: it covers the blocks structure detection dropped
    # because they are zero.  A perturbation inside such a block changes A only for a plan
    # that keeps every block, so the differences use the reference work model (structure none).
    full = asgkron.Plan.create(mats, idx, 4, structure="none")
    for t, a, b in picks[:32]:
        gval = G[t][t][a, b].item()
        mp = [[m.copy() for m in row] for row in mats]
        mm = [[m.copy() for m in row] for row in mats]
        mp[t][t][a, b] += h
        mm[t][t][a, b] -= h
        full.update_ops(mp)
        yp = full.apply(ft)
        full.update_ops(mm)
        ym = full.apply(ft)
        fd = dloss(yp, ym) / (2 * h)
        assert abs(fd - gval) <= 1e-6 * max(1.0, abs(gval)), (t, a, b, fd, gval)
    full.close()
    # FP32 forward + backward within 1e-6 / 1e-5 of FP64
    r32 = plan.apply(ft.float()) - yst.float()
    fbar32 = plan.apply_T(r32)
    torch.cuda.synchronize()
    assert rel2(fbar32.double().cpu().numpy(), fb) <= 1e-5


def test_autograd_harness(dev):
    import asgkron
    from asgkron.api import autograd_apply

    _, _, idx, mats = problem("continuity3", 3, 3)
    plan = asgkron.Plan.create(mats, idx, 3)
    n = plan.dof
    rng = np.random.default_rng(1)
    f = _t(rng.standard_normal(n), dev).requires_grad_(True)
    ops = [[_t(np.asarray(m), dev).requires_grad_(True) for m in row] for row in mats]
    ys = _t(rng.standard_normal(n), dev)
    y = autograd_apply(plan, f, ops)
    L = 0.5 * torch.sum((y - ys) ** 2)
    L.backward()
    r = (plan.apply(f.detach()) - ys)
    assert torch.allclose(f.grad, plan.apply_T(r), rtol=1e-13, atol=1e-13)
    G = plan.grad_ops(f.detach(), r)
    active = plan.active_factors()
    for t in range(3):
        for d in range(3):
            if active[t][d]:
                assert torch.allclose(ops[t][d].grad, G[t][d], rtol=1e-13, atol=1e-13)
            else:
                assert float(ops[t][d].grad.abs().max()) == 0.0
    # the adjoint kernels are deterministic
    assert torch.equal(plan.apply_T(r), plan.apply_T(r))
