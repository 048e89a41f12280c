"""Kronmult path: kronmultN_batch lists, their GPU execution, gemm_vbatched and krond.

Follows Kronmult/test1_batch.m: factors A1 2x3, A2 3x4, A3 4x5, A4 5x6, A5 6x7, A6 3x2,
nvec = 2, result against the explicit kron with tol = 1e-7 * numel (seeded here)."""
import numpy as np
import pytest

from oracle import asgard_oracle as O

SHAPES = [(2, 3), (3, 4), (4, 5), (5, 6), (6, 7), (3, 2)]


def _mats(n, seed=11):
    rng = np.random.default_rng(seed)
    return [rng.random(s) for s in SHAPES[:n]], rng


@pytest.mark.parametrize("n", range(1, 7))
def test_batch_lists_match_oracle(n):
    """The planner records the same GEMMs, level by level, as kronmult{n}_batch.m (CPU only)."""
    from asgkron.kron import KronPlan

    mats, rng = _mats(n)
    nc = int(np.prod([m.shape[1] for m in mats]))
    X = rng.random((nc, 2))
    lists = [O.BatchList() for _ in range(n)]
    O.kronmult_batch(mats, X, lists)
    ref = [(L + 1, e["m"], e["n"], e["k"], e["transA"], e["transB"]) for L, bl in enumerate(lists) for e in bl.entries]
    plan = KronPlan([m.shape for m in mats], 2)
    got = [(d["level"], d["m"], d["n"], d["k"], d["trans_a"], d["trans_b"]) for d in plan.lists()]
    assert sorted(got) == sorted(ref)
    # every level-L list is executed after all lists < L (the planner's order)
    lv = [d["level"] for d in plan.lists()]
    assert lv == sorted(lv)
    plan.close()


def test_flop_model_matches_oracle():
    from asgkron.kron import KronPlan

    for n in range(2, 7):
        mats, _ = _mats(n)
        nr = [m.shape[0] for m in mats]
        nc = [m.shape[1] for m in mats]
        f1, f2, meth, _, _ = O.flops_kron(nr, nc)
        plan = KronPlan(list(zip(nr, nc)), 1)
        total = sum(2.0 * d["m"] * d["n"] * d["k"] for d in plan.lists())
        assert total == pytest.approx(min(f1, f2) if meth == (1 if f1 <= f2 else 2) else f1)
        plan.close()


def test_plan_rejects_bad_sizes():
    from asgkron._lib import AsgError
    from asgkron.kron import KronPlan

    with pytest.raises(AsgError, match="nkron=7"):
        KronPlan([(2, 2)] * 7, 1)
    with pytest.raises(AsgError, match="size 0x2"):
        KronPlan([(0, 2)], 1)


# ------------------------------------------------------------------------------------- GPU
torch = pytest.importorskip("torch")


def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


@pytest.mark.gpu
@pytest.mark.parametrize("n", range(1, 7))
def test_kronmult_batch_gpu_vs_kron(n):
    _gpu()
    from asgkron.kron import kronmult_batch

    mats, rng = _mats(n)
    nc = int(np.prod([m.shape[1] for m in mats]))
    X = rng.random((nc, 2))
    lists, Y = kronmult_batch(mats, X)
    Yok = O.krond(mats) @ X
    assert np.max(np.abs(Y - Yok)) < 1e-7 * Yok.size
    np.testing.assert_allclose(Y, Yok, rtol=1e-12, atol=1e-12)
    # each recorded GEMM is consistent with its operands (C = op(A) op(B))
    for bl in lists:
        for e in bl:
            opA = e["A"].T if e["transA"] == "T" else e["A"]
            opB = e["B"].T if e["transB"] == "T" else e["B"]
            np.testing.assert_allclose(e["C"], opA @ opB, rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
def test_kron_multd_gpu_deg4_d6():
    _gpu()
    from asgkron.kron import kron_multd

    rng = np.random.default_rng(3)
    mats = [rng.standard_normal((4, 4)) for _ in range(6)]
    X = rng.standard_normal((4096, 3))
    Y = kron_multd(6, mats, X)
    np.testing.assert_allclose(Y, O.kron_multd(6, mats, X), rtol=1e-12, atol=1e-11)


@pytest.mark.gpu
def test_kron_batch_fp32_matches_fp64():
    _gpu()
    from asgkron.kron import KronPlan, _dev

    rng = np.random.default_rng(5)
    mats = [rng.standard_normal((4, 4)) for _ in range(4)]
    X = rng.standard_normal((256, 8))
    p = KronPlan([m.shape for m in mats], 8)
    y64 = p.apply([_dev(m, np.float64) for m in mats], _dev(X, np.float64))
    y32 = p.apply([_dev(m, np.float32) for m in mats], _dev(X, np.float32))
    torch.cuda.synchronize()
    a, b = y64.cpu().numpy(), y32.double().cpu().numpy()
    assert np.linalg.norm(a - b) / np.linalg.norm(a) < 1e-6


@pytest.mark.gpu
def test_gemm_vbatched_uses_klist():
    """gemm_vbatched.m:25 reads kk from nlist; the C ABI reads klist (documented fix)."""
    _gpu()
    from asgkron.kron import gemm_vbatched

    rng = np.random.default_rng(7)
    ms, ns, ks = [3, 5, 2, 7], [4, 1, 6, 2], [2, 3, 5, 1]
    for ta, tb in (("N", "N"), ("T", "N"), ("N", "T"), ("T", "T")):
        A = [rng.standard_normal((k, m) if ta == "T" else (m, k)) for m, k in zip(ms, ks)]
        B = [rng.standard_normal((n, k) if tb == "T" else (k, n)) for n, k in zip(ns, ks)]
        Cin = [rng.standard_normal((m, n)) for m, n in zip(ms, ns)]
        got = gemm_vbatched(ta, tb, ms, ns, ks, 1.5, A, B, -0.5, Cin)
        want = O.gemm_vbatched(ta, tb, ms, ns, ks, 1.5, A, B, -0.5, Cin)
        for g, w in zip(got, want):
            np.testing.assert_allclose(g, w, rtol=1e-13, atol=1e-13)


@pytest.mark.gpu
def test_krond_gpu():
    _gpu()
    from asgkron.kron import krond

    mats, _ = _mats(4)
    np.testing.assert_allclose(krond(4, mats), O.krond(mats), rtol=1e-15, atol=0)
