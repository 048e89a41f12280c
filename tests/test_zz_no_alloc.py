"""asg_kron_batch_static_f64: the Kronecker executor that allocates nothing, against the
workspace-taking asg_kron_batch_f64 on the same plan and inputs.

Collected last on purpose: it must hold both in a fresh process and after every other test
has used the library (the static scratch then holds whatever earlier calls left there)."""
import ctypes as C

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

LIMIT = 8 << 20  # ASG_KRON_STATIC_SCRATCH_BYTES
ASG_ERR_CAPACITY = 6

CASES = [
    ([(4, 4)] * 6, 3),                                          # a deg-4 d-6 element block, method 1
    ([(2, 3), (3, 4), (4, 5), (5, 6), (6, 7), (3, 2)], 2),      # Kronmult/test1_batch.m shapes
    ([(5, 3), (2, 7), (6, 6)], 130),                            # method 2 at the top, 390 GEMMs on one level
    ([(7, 2), (3, 9), (2, 5), (6, 3)], 70),                     # mixed methods, several launches per level
]


def _static(plan, A, X, Y):
    from asgkron._lib import lib

    ptrs = (C.c_void_p * plan.n)(*[a.data_ptr() for a in A])
    s = torch.cuda.current_stream()
    return lib().asg_kron_batch_static_f64(plan._h, ptrs, C.c_void_p(X.data_ptr()), C.c_void_p(Y.data_ptr()),
                                           C.c_void_p(s.cuda_stream))


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


@pytest.mark.parametrize("case", range(len(CASES)))
def test_static_matches_workspace_entry(dev, case):
    from asgkron.kron import KronPlan, _dev

    shapes, nvec = CASES[case]
    plan = KronPlan(shapes, nvec)
    assert 0 < plan.work_bytes[8] <= LIMIT
    rng = np.random.default_rng(100 + case)
    A = [_dev(rng.standard_normal(s), np.float64) for s in shapes]
    for call in range(2):  # two calls in a row; the second sees the first one's temporaries
        X = _dev(rng.standard_normal((plan.cols, nvec)), np.float64)
        want = plan.apply(A, X)
        got = torch.full_like(want, float("nan"))
        assert _static(plan, A, X, got) == 0
        torch.cuda.synchronize()
        torch.testing.assert_close(got, want, rtol=1e-13, atol=1e-13)
    plan.close()


def test_static_rejects_plans_beyond_the_scratch(dev):
    from asgkron._lib import last_error
    from asgkron.kron import KronPlan

    plan = KronPlan([(8, 8)] * 6, 8)
    assert plan.work_bytes[8] > LIMIT
    X = torch.zeros(plan.cols * 8, dtype=torch.float64, device=dev)
    Y = torch.zeros(plan.rows * 8, dtype=torch.float64, device=dev)
    A = [torch.zeros(64, dtype=torch.float64, device=dev) for _ in range(6)]
    assert _static(plan, A, X, Y) == ASG_ERR_CAPACITY
    msg = last_error()
    assert "static scratch holds 8388608" in msg and str(plan.work_bytes[8]) in msg
    plan.close()
