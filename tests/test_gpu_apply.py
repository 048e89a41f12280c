"""apply_A on the GPU through the C ABI, against the CPU oracle (apply_A.m:102-236).

Tolerances: FP64 kernels <= 1e-12 relative 2-norm (the reference parity bound); FP32 kernels
(Kahan-compensated across the column reduction) <= 1e-6 relative to FP64.
"""
import numpy as np
import pytest

from cases import problem, random_problem, rel2
from oracle import asgard_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

FP64_TOL = 1e-12
FP32_TOL = 1e-6


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


def _plan(mats, idx, deg, **kw):
    import asgkron

    return asgkron.Plan.create(mats, idx, deg, **kw)


def _apply(plan, f, dev, dtype=torch.float64):
    ft = torch.from_numpy(np.asarray(f)).to(dev, dtype)
    y = plan.apply(ft)
    torch.cuda.synchronize()
    return y.double().cpu().numpy()


@pytest.mark.parametrize("structure", ["none", "detect"])
@pytest.mark.parametrize("conn", [False, True])
def test_continuity2_lev4_deg2_vs_oracle_loop(dev, structure, conn):
    """The CPU-runnable configuration: continuity2, SG lev 4, deg 2 (48 elements, 192 DOF)."""
    import asgkron

    pde, table, idx, mats = problem("continuity2", 4, 2)
    f = np.random.default_rng(0).standard_normal(idx.shape[0] * 4)
    pairs = None
    conn_cells = None
    if conn:
        rp, cols = asgkron.connect_nD(table, 4, 4)
        pairs = (rp, cols + 1)
        conn_cells = asgkron.connectivity_cells(rp, cols)
    want = O.apply_A_loop(mats, idx.astype(np.int64), 2, f, conn=conn_cells)
    plan = _plan(mats, idx, 2, pairs=pairs, structure=structure)
    assert rel2(_apply(plan, f, dev), want) <= FP64_TOL
    assert rel2(_apply(plan, f, dev, torch.float32), want) <= FP32_TOL
    st = plan.stats()
    assert st["num_pairs"] == (2304 if not conn else rp[-1])
    if structure == "none":
        assert st["num_entries"] == st["num_pairs"] * 2


def test_continuity3_lev6_deg3_precision(dev):
    """Precision configuration: continuity3, SG lev 6, deg 3 (688 elements, 18,576 DOF), f~N(0,1) seed 1."""
    pde, table, idx, mats = problem("continuity3", 6, 3)
    assert idx.shape[0] == 688
    f = np.random.default_rng(1).standard_normal(idx.shape[0] * 27)
    rows = np.arange(0, 688, 7)
    want = O.apply_A_rows(mats, idx.astype(np.int64), 3, f, rows=rows)
    B = 27
    for structure in ("none", "detect"):
        plan = _plan(mats, idx, 3, structure=structure)
        y64 = _apply(plan, f, dev)
        y32 = _apply(plan, f, dev, torch.float32)
        got = y64.reshape(-1, B)[rows].ravel()
        assert rel2(got, want) <= FP64_TOL, structure
        assert rel2(y32, y64) <= FP32_TOL, structure


def test_diffusion2_lev8_deg4(dev):
    """Implicit configuration's operator: diffusion2 LDG, SG lev 8, deg 4 (1,280 elements)."""
    pde, table, idx, mats = problem("diffusion2", 8, 4)
    assert idx.shape[0] == 1280
    f = np.random.default_rng(2).standard_normal(idx.shape[0] * 16)
    rows = np.arange(0, 1280, 37)
    want = O.apply_A_rows(mats, idx.astype(np.int64), 4, f, rows=rows)
    for structure in ("none", "detect"):
        plan = _plan(mats, idx, 4, structure=structure)
        y64 = _apply(plan, f, dev)
        assert rel2(y64.reshape(-1, 16)[rows].ravel(), want) <= FP64_TOL, structure
        assert rel2(_apply(plan, f, dev, torch.float32), y64) <= FP32_TOL


def test_continuity6_lev4_deg4_kernels_agree(dev):
    """Differentiation-scale configuration: continuity6, SG lev 4, deg 4 (501 elements of 4096).

    Sampled rows against the oracle; the single-mode fiber kernel, the CTA chain kernel on
    the same structured work list, and the reference work model (every pair x term, full
    6-mode chain) agree."""
    import asgkron

    pde, table, idx, mats = problem("continuity6", 4, 4)
    assert idx.shape[0] == 501
    B = 4096
    f = np.random.default_rng(4).standard_normal(idx.shape[0] * B)
    rows = np.array([0, 1, 77, 250, 500])
    want = O.apply_A_rows(mats, idx.astype(np.int64), 4, f, rows=rows)
    p = _plan(mats, idx, 4, structure="detect")
    st = p.stats()
    assert st["kernel_kind"] == asgkron._lib.KERNEL_SINGLE_TMA
    assert st["active_modes_max"] == 1
    y_single = _apply(p, f, dev)
    assert p.device_status() == 0
    assert rel2(y_single.reshape(-1, B)[rows].ravel(), want) <= FP64_TOL
    y32 = _apply(p, f, dev, torch.float32)
    assert p.device_status() == 0
    assert rel2(y32, y_single) <= FP32_TOL
    # the streaming kernel: FP32 within tolerance, bitwise repeatable; its FP64 is kind 3's
    p.set_kernel(asgkron._lib.KERNEL_STREAM)
    y_stream = _apply(p, f, dev, torch.float32)
    assert p.device_status() == 0
    assert rel2(y_stream, y_single) <= FP32_TOL
    assert np.array_equal(_apply(p, f, dev, torch.float32), y_stream)
    assert np.array_equal(_apply(p, f, dev), y_single)
    # the persistent row-list kernel runs kind 3's arithmetic per row: bitwise equal
    p.set_kernel(5)
    assert np.array_equal(_apply(p, f, dev), y_single)
    assert np.array_equal(_apply(p, f, dev, torch.float32), y32)
    assert p.device_status() == 0
    # two tiles per consumer thread: kind 3's operations per value, bitwise equal in FP32;
    # its FP64 side is kind 3
    p.set_kernel(asgkron._lib.KERNEL_SINGLE_TMA_X2)
    assert np.array_equal(_apply(p, f, dev, torch.float32), y32)
    assert np.array_equal(_apply(p, f, dev), y_single)
    assert p.device_status() == 0
    for kind in (asgkron._lib.KERNEL_SINGLE_TMA3, asgkron._lib.KERNEL_SINGLE_MODE):
        p.set_kernel(kind)
        assert rel2(_apply(p, f, dev), y_single) <= FP64_TOL
        assert rel2(_apply(p, f, dev, torch.float32), y_single) <= FP32_TOL
        assert p.device_status() == 0
    p.set_kernel(asgkron._lib.KERNEL_CHAIN_CTA)
    y_chain = _apply(p, f, dev)
    assert rel2(y_chain, y_single) <= FP64_TOL
    assert rel2(_apply(p, f, dev, torch.float32), y_single) <= FP32_TOL
    pn = _plan(mats, idx, 4, structure="none")
    assert pn.stats()["num_entries"] == 501 * 501 * 6
    y_none = _apply(pn, f, dev)
    assert rel2(y_none, y_single) <= FP64_TOL


@pytest.mark.parametrize("name,lev,deg,kinds", [("continuity6", 3, 4, [3, 4, 5, 7, 8, 2, 1]),
                                               ("continuity2", 4, 2, [6, 0, 1]), ("continuity3", 4, 3, [6, 0, 1])])
def test_apply_residual_equals_apply_minus_ystar(dev, name, lev, deg, kinds):
    """asg_apply_residual_*: r = A f - y* equals the apply followed by a subtraction in the same
    precision, bitwise, for every kernel family the plan can run (subtracted in the apply's
    own stores for kinds 2-5, 7, 8; a second launch for kinds 0, 1, 6), in both precisions."""
    import asgkron

    pde, table, idx, mats = problem(name, lev, deg)
    p = _plan(mats, idx, deg)
    rng = np.random.default_rng(5)
    f, ys = rng.standard_normal(p.dof), rng.standard_normal(p.dof)
    for kind in kinds:
        p.set_kernel(kind)
        for dt in (torch.float64, torch.float32):
            ft, yst = torch.from_numpy(f).to(dev, dt), torch.from_numpy(ys).to(dev, dt)
            want = p.apply(ft) - yst
            r = p.apply_residual(ft, yst)
            torch.cuda.synchronize()
            assert torch.equal(r, want), (kind, dt)
    assert p.device_status() == 0
    with pytest.raises(asgkron.AsgError):
        p.apply_residual(ft, yst, yst)  # r must not alias ystar


@pytest.mark.parametrize("name,lev,deg", [("continuity2", 4, 2), ("continuity2", 3, 4), ("continuity3", 4, 3),
                                          ("continuity3", 3, 4), ("diffusion2", 5, 4), ("continuity6", 2, 2),
                                          ("continuity3", 2, 6)])
def test_small_block_single_mode_kernel(dev, name, lev, deg):
    """Small blocks (deg^d <= 256) with one applied factor per term run the grouped-lane kernel
    by default: FP64 against the oracle, against the warp chain kernel, FP32 against FP64,
    and bitwise repeatable."""
    import asgkron

    pde, table, idx, mats = problem(name, lev, deg)
    N, D = idx.shape
    B = deg ** D
    f = np.random.default_rng(lev * 10 + deg).standard_normal(N * B)
    p = _plan(mats, idx, deg)
    assert p.stats()["kernel_kind"] == 6
    y = _apply(p, f, dev)
    assert np.array_equal(_apply(p, f, dev), y)
    rows = np.arange(0, N, max(1, N // 6))
    want = O.apply_A_rows(mats, idx.astype(np.int64), deg, f, rows=rows)
    assert rel2(y.reshape(-1, B)[rows].ravel(), want) <= FP64_TOL
    assert rel2(_apply(p, f, dev, torch.float32), y) <= FP32_TOL
    p.set_kernel(asgkron._lib.KERNEL_CHAIN_WARP)
    assert rel2(_apply(p, f, dev), y) <= FP64_TOL


@pytest.mark.parametrize("lev", [2, 3])
def test_continuity6_small_levels_row_lists(dev, lev):
    """continuity6 deg 4 at levels with fewer elements than resident CTAs (one row per CTA)
    and with several rows per CTA: the streaming kernel (kind 7) agrees with kind 3 in FP32,
    kinds 3, 5 and 8 agree bitwise, FP64 matches the oracle."""
    pde, table, idx, mats = problem("continuity6", lev, 4)
    N = idx.shape[0]
    f = np.random.default_rng(lev).standard_normal(N * 4096)
    p = _plan(mats, idx, 4, structure="detect")
    p.set_kernel(7)
    y_stream = _apply(p, f, dev, torch.float32)
    assert p.device_status() == 0
    p.set_kernel(3)
    y3 = _apply(p, f, dev)
    y3s = _apply(p, f, dev, torch.float32)
    assert rel2(y_stream, y3) <= FP32_TOL
    p.set_kernel(5)
    assert np.array_equal(_apply(p, f, dev), y3)
    assert np.array_equal(_apply(p, f, dev, torch.float32), y3s)
    assert p.device_status() == 0
    p.set_kernel(8)
    assert np.array_equal(_apply(p, f, dev, torch.float32), y3s)
    assert p.device_status() == 0
    rows = np.arange(0, N, max(1, N // 5))
    want = O.apply_A_rows(mats, idx.astype(np.int64), 4, f, rows=rows)
    assert rel2(y3.reshape(-1, 4096)[rows].ravel(), want) <= FP64_TOL


@pytest.mark.parametrize("d,lev,deg", [(2, 3, 2), (2, 4, 4), (3, 3, 3), (3, 4, 2), (4, 3, 2), (4, 3, 3), (1, 5, 4),
                                       (5, 2, 2), (6, 2, 2)])
def test_random_dense_operators_vs_oracle(dev, d, lev, deg):
    """Batched configuration's operator model (dense random N(0,1/deg) factors): no structure,
    every pair and term runs the full chain."""
    table, idx, mats = random_problem(3 + d * 10 + lev, d, lev, deg)
    N = idx.shape[0]
    f = np.random.default_rng(5).standard_normal(N * deg ** d)
    rows = np.arange(0, N, max(1, N // 16))
    want = O.apply_A_rows(mats, idx.astype(np.int64), deg, f, rows=rows)
    plan = _plan(mats, idx, deg, structure="detect")
    y = _apply(plan, f, dev)
    B = deg ** d
    assert rel2(y.reshape(-1, B)[rows].ravel(), want) <= FP64_TOL
    assert rel2(_apply(plan, f, dev, torch.float32), y) <= FP32_TOL


def test_deterministic_linear_and_host_path(dev):
    pde, table, idx, mats = problem("continuity3", 4, 3)
    plan = _plan(mats, idx, 3)
    rng = np.random.default_rng(9)
    n = idx.shape[0] * 27
    f1, f2 = rng.standard_normal(n), rng.standard_normal(n)
    a = _apply(plan, f1, dev)
    b = _apply(plan, f1, dev)
    assert np.array_equal(a, b)  # no atomics: bitwise reproducible
    c = _apply(plan, f1 + 2.5 * f2, dev)
    assert rel2(c, a + 2.5 * _apply(plan, f2, dev)) <= 1e-14
    h = plan.apply_host(f1)
    assert np.array_equal(h, a)
    h32 = plan.apply_host(f1.astype(np.float32))
    assert h32.dtype == np.float32 and rel2(h32, a) <= FP32_TOL


@pytest.mark.parametrize("name,lev,deg,kind", [("continuity3", 4, 3, None), ("continuity6", 2, 4, None),
                                              ("continuity6", 3, 4, None), ("continuity6", 4, 4, None),
                                              ("continuity6", 4, 4, 5), ("continuity6", 4, 4, 8)])
def test_host_path_pinned_output(dev, name, lev, deg, kind):
    """A page-locked y is written by the apply kernel itself (no device-to-host copy); the
    result equals the pageable copy path and the device apply bitwise, in both precisions.
    continuity6 plans take the chunked host path (f in by element chunks, each chunk's ready
    rows launched as it lands), including when the plan runs kind 5 or 8 on the device; a
    page-locked f arrives in the gathered order (longest rows' columns first), a pageable one
    by contiguous chunks, with the same result."""
    pde, table, idx, mats = problem(name, lev, deg)
    plan = _plan(mats, idx, deg)
    if kind is not None:
        plan.set_kernel(kind)
    f = np.random.default_rng(21).standard_normal(plan.dof)
    for dt in (torch.float64, torch.float32):
        fh = torch.from_numpy(f).to(dt).pin_memory()
        yh = torch.full_like(fh, float("nan")).pin_memory()
        plan.apply_host(fh.numpy(), yh.numpy())
        pageable = plan.apply_host(fh.numpy().copy())
        assert np.array_equal(yh.numpy(), pageable)
        assert np.array_equal(plan.apply_host(fh.numpy()), pageable)  # page-locked f (gathered), pageable y
        assert np.array_equal(yh.numpy(), _apply(plan, f, dev, dt).astype(yh.numpy().dtype))
        for _ in range(4):  # repeated buffers: direct, captured into a graph, then replayed
            yh.fill_(float("nan"))
            plan.apply_host(fh.numpy(), yh.numpy())
            assert np.array_equal(yh.numpy(), pageable)
        fh.copy_(torch.from_numpy(-f).to(dt))  # new values in the same buffers
        plan.apply_host(fh.numpy(), yh.numpy())
        assert np.array_equal(yh.numpy(), -pageable)
    assert plan.device_status() == 0


def test_apply_A_matlab_mirror(dev):
    """asgkron.apply_A keeps apply_A.m's signature: pde.terms{t}.terms_1D{d}.mat, opts,
    A_data.element_local_index_D, f, deg; use_connectivity picks pde.connectivity."""
    import asgkron

    pde, table, idx, mats = problem("continuity2", 4, 2)
    A_data = asgkron.global_matrix(table)
    terms = [{"terms_1D": [{"mat": m} for m in row], "imex": "N"} for row in mats]
    rp, cols = asgkron.connect_nD(table, 4, 4)
    pde_obj = {"terms": terms, "connectivity": asgkron.connectivity_cells(rp, cols)}
    f = np.random.default_rng(0).standard_normal(idx.shape[0] * 4)
    want = O.apply_A_loop(mats, idx.astype(np.int64), 2, f)
    got = asgkron.apply_A(pde_obj, {"use_connectivity": False}, A_data, f, 2)
    assert rel2(got, want) <= FP64_TOL
    got_c = asgkron.apply_A(pde_obj, {"use_connectivity": True}, A_data, f, 2)
    want_c = O.apply_A_loop(mats, idx.astype(np.int64), 2, f, conn=pde_obj["connectivity"])
    assert rel2(got_c, want_c) <= FP64_TOL
    # imex filter: no 'E' terms -> zero
    assert not np.any(asgkron.apply_A(pde_obj, {}, A_data, f, 2, imex_flag="E"))
    asgkron.clear_plan_cache()


def test_apply_A_matlab_mirror_build_A(dev):
    """[ftmp, A, ALHS] = apply_A(...): A and ALHS (a non-identity LHS mass term) equal the
    oracle's krond assembly (apply_A.m:170-180,209-221), dense and sparse, over all pairs and
    over pde.connectivity; ALHS is 0 without LHS terms (apply_A.m:55)."""
    import asgkron

    pde, table, idx, mats = problem("continuity2", 3, 2)
    A_data = asgkron.global_matrix(table)
    rng = np.random.default_rng(3)
    lhs = [[np.eye(m.shape[0]) + 0.1 * rng.standard_normal(m.shape) for m in mats[0]]]
    rp, cols = asgkron.connect_nD(table, 3, 3)
    pde_obj = {"terms": [{"terms_1D": [{"mat": m} for m in row], "imex": "N"} for row in mats],
               "termsLHS": [{"terms_1D": [{"mat": m} for m in lhs[0]]}],
               "connectivity": asgkron.connectivity_cells(rp, cols)}
    f = rng.standard_normal(idx.shape[0] * 4)
    for conn in (False, True):
        cc = pde_obj["connectivity"] if conn else None
        want_y = O.apply_A_loop(mats, idx.astype(np.int64), 2, f, conn=cc)
        _, want_A = O.apply_A_loop(mats, idx.astype(np.int64), 2, f, conn=cc, build_A=True)
        _, want_L = O.apply_A_loop(lhs, idx.astype(np.int64), 2, f, conn=cc, build_A=True)
        for sparse in (False, True):
            y, A, AL = asgkron.apply_A(pde_obj, {"use_connectivity": conn, "use_sparse_A": sparse}, A_data, f, 2,
                                       nargout=3)
            Ad, ALd = (A.toarray(), AL.toarray()) if sparse else (A, AL)
            assert rel2(y, want_y) <= FP64_TOL
            assert rel2(Ad @ f, y) <= FP64_TOL
            assert np.abs(Ad - want_A).max() <= 1e-12 * np.abs(want_A).max()
            assert np.abs(ALd - want_L).max() <= 1e-12 * np.abs(want_L).max()
    no_lhs = {"terms": pde_obj["terms"]}
    y, A, AL = asgkron.apply_A(no_lhs, {}, A_data, f, 2, nargout=3)
    assert isinstance(AL, int) and AL == 0
    asgkron.clear_plan_cache()


def test_argument_errors(dev):
    import asgkron
    from asgkron._lib import AsgError

    pde, table, idx, mats = problem("continuity2", 3, 2)
    plan = _plan(mats, idx, 2)
    f = torch.zeros(plan.dof + 1, dtype=torch.float64, device=dev)
    with pytest.raises(AsgError, match="16-byte aligned"):
        import ctypes as C

        asgkron.lib().asg_apply_f64  # noqa
        from asgkron._lib import check

        check(asgkron.lib().asg_apply_f64(plan.handle, C.c_void_p(f.data_ptr() + 8), C.c_void_p(f.data_ptr()), None))
    bad = idx.copy()
    bad[3, 0] = 0  # below the 1-based index base
    with pytest.raises(AsgError, match="index base"):
        _plan(mats, bad, 2)
    small = [[m[:4, :4] for m in row] for row in mats]
    with pytest.raises(AsgError, match="ld="):
        _plan(small, idx, 2)


@pytest.mark.parametrize("name,lev,deg", [("continuity6", 3, 4), ("continuity3", 4, 3), ("continuity2", 4, 2)])
def test_tuner_choice_matches_default(dev, name, lev, deg):
    """asg_plan_tune times the kernel families of the plan per precision and keeps the fastest:
    the tuned plan's results equal the default's within the precision's tolerance (FP64 against
    the oracle's rows as well), and set_kernel clears the choice."""
    import asgkron

    pde, table, idx, mats = problem(name, lev, deg)
    N = idx.shape[0]
    B = deg ** idx.shape[1]
    f = np.random.default_rng(3).standard_normal(N * B)
    p = _plan(mats, idx, deg)
    y64, y32 = _apply(p, f, dev), _apply(p, f, dev, torch.float32)
    default = p.stats()["kernel_kind"]
    for dtype in (torch.float64, torch.float32):
        r = p.tune(dtype)
        assert r["ms"] > 0 and r["ms"] <= r["default_ms"] * 1.0001 and p.kernel_for(dtype) == r["kind"]
    assert p.device_status() == 0
    t64, t32 = _apply(p, f, dev), _apply(p, f, dev, torch.float32)
    assert rel2(t64, y64) <= FP64_TOL and rel2(t32, y32) <= FP32_TOL and rel2(t32, t64) <= FP32_TOL
    rows = np.arange(0, N, max(1, N // 5))
    want = O.apply_A_rows(mats, idx.astype(np.int64), deg, f, rows=rows)
    assert rel2(t64.reshape(N, B)[rows].ravel(), want) <= FP64_TOL
    p.set_kernel(default)
    assert p.kernel_for(torch.float64) in (default, asgkron._lib.KERNEL_SINGLE_TMA)
    p.close()
