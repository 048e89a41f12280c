"""The MEX gateways (dg-sparsegrid_gb300/mex/) compile against a stand-in mex.h with
-Wall -Werror and run their argument checks on a host without a GPU: errors come back as
mexErrMsgIdAndTxt ids in the reference's "name: reason" style (kron_multd.m:7-12,
kronmult6_batch.m:30-35); a well-formed call reaches the library, whose failure to find a
device is reported as asgkron:apply instead of crashing MATLAB."""
import numpy as np
import pytest

import mexharness as M
from cases import problem

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module")
def gw():
    return {name: M.Gateway(name) for name in ("apply_A_mex", "apply_A_T_mex")}


@pytest.fixture(scope="module")
def c2():
    pde, table, idx, mats = problem("continuity2", 3, 2)
    return [[m for m in row] for row in mats], idx.astype(np.float64)


def _err(g, nlhs, *args):
    with pytest.raises(M.MexError) as e:
        g.call(nlhs, *args)
    return e.value


def test_gateways_compile_and_check_arguments(gw, c2):
    ops, idx = c2
    N = idx.shape[0]
    f = np.zeros(N * 4)
    a, t = gw["apply_A_mex"], gw["apply_A_T_mex"]
    e = _err(a, 1, ops, idx, 2)
    assert e.ident == "asgkron:args" and e.msg.startswith("apply_A_mex: expected")
    e = _err(t, 1, ops, idx, 2, f)
    assert e.ident == "asgkron:args" and e.msg.startswith("apply_A_T_mex: expected")
    e = _err(a, 2, ops, idx, 2, f)
    assert e.ident == "asgkron:args" and "one output" in e.msg
    e = _err(t, 3, ops, idx, 2, f, f)
    assert e.ident == "asgkron:args" and "two outputs" in e.msg
    e = _err(a, 1, np.eye(3), idx, 2, f)
    assert "ops must be a T x d cell" in e.msg
    e = _err(a, 1, ops, idx[:, :1], 2, f)
    assert "idx1d must be a real double N x d" in e.msg
    e = _err(a, 1, ops, idx, 2.5, f)
    assert "deg must be a positive integer" in e.msg
    bad = [[m for m in row] for row in ops]
    bad[1][0] = ops[1][0][:, :-1]
    e = _err(a, 1, bad, idx, 2, f)
    assert "square real double" in e.msg
    e = _err(a, 1, ops, idx, 2, f, np.zeros(3), np.zeros(2))
    assert "row_ptr must hold N+1 offsets" in e.msg


def test_wellformed_call_reports_library_failure(gw, c2):
    if torch.cuda.is_available():
        pytest.skip("checks the no-device path")
    ops, idx = c2
    f = np.zeros(idx.shape[0] * 4)
    e = _err(gw["apply_A_mex"], 1, ops, idx, 2, f)
    assert e.ident == "asgkron:apply" and e.msg.startswith("apply_A_mex:") and "status" in e.msg
    e = _err(gw["apply_A_T_mex"], 2, ops, idx, 2, f, f)
    assert e.ident == "asgkron:apply" and e.msg.startswith("apply_A_T_mex:")
    assert not gw["apply_A_mex"].L.stub_locked()  # no plan was cached
