"""GPU time steppers: RK3 against the reference's gold trajectories and the oracle; backward
Euler (mixed-precision GMRES + iterative refinement) against a direct solve."""
import os

import numpy as np
import pytest

from cases import rel2
from oracle import asgard_oracle as O

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu
G = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def dev():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch.device("cuda:0")


@pytest.mark.parametrize("name,pdename,lev,deg", [("continuity2_sg_l4_d3", "continuity2", 4, 3),
                                                  ("continuity3_sg_l4_d3", "continuity3", 4, 3),
                                                  ("continuity2_sg_l2_d2", "continuity2", 2, 2)])
@pytest.mark.parametrize("graph", [False, True, "queued"])
def test_rk3_matches_gold_trajectory(dev, name, pdename, lev, deg, graph):
    """5 RK3 steps at CFL 0.01 on the GPU reproduce gold/generated-inputs/time_advance (central
    flux, operators built at max_lev 8, sources without the mass solve, as the gold was made).
    "queued" replays the five captured steps without waiting in between: each step's time
    factors must reach the device unchanged by the later steps' uploads."""
    import asgkron
    from asgkron import pdes
    from asgkron.steppers import RK3Stepper

    pde = getattr(pdes, pdename)(lev, 0.0)
    table = asgkron.hash_table_sparse_nD(pde.levels, 8)
    idx = table.idx1d()
    mats = pde.term_mats(deg, construction_level=8)
    plan = asgkron.Plan.create(mats, idx, deg)
    st = RK3Stepper(plan, pde, idx)
    f = torch.from_numpy(pde.initial_condition(deg, idx)).to(dev)
    dt = pde.dt(0.01)
    gold = np.load(os.path.join(G, "time_advance.npz"))
    if graph:
        st.capture(f, dt)
    if graph == "queued":
        for i in range(5):
            st.replay(i * dt)
        torch.cuda.synchronize()
        assert rel2(f.cpu().numpy(), gold["%s_t4" % name]) <= 1e-13
        return
    for i in range(5):
        if graph:
            st.replay(i * dt)
        else:
            st.step(f, i * dt, dt)
        torch.cuda.synchronize()
        g = gold["%s_t%d" % (name, i)]
        assert rel2(f.cpu().numpy(), g) <= 1e-13, i


def test_lincomb_matches_host_sum(dev):
    """asg_lincomb_f64: sum_s coef[s] * vecs[s] (the separable sources of source_vector.m)
    against the same sum on the host, to round-off; ns = 0 gives zeros."""
    import ctypes as C

    from asgkron._lib import check, lib

    rng = np.random.default_rng(11)
    n, ns = 1000, 3
    vecs = [torch.from_numpy(rng.standard_normal(n)).to(dev) for _ in range(ns)]
    ptrs = torch.tensor([v.data_ptr() for v in vecs], dtype=torch.int64, device=dev)
    coef = torch.from_numpy(rng.standard_normal(ns)).to(dev)
    out = torch.full((n,), float("nan"), dtype=torch.float64, device=dev)
    s = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    check(lib().asg_lincomb_f64(n, ns, C.c_void_p(coef.data_ptr()), C.c_void_p(ptrs.data_ptr()),
                                C.c_void_p(out.data_ptr()), s))
    torch.cuda.synchronize()
    want = sum(c * v for c, v in zip(coef.cpu().numpy(), [v.cpu().numpy() for v in vecs]))
    assert rel2(out.cpu().numpy(), want) <= 1e-15
    check(lib().asg_lincomb_f64(n, 0, None, None, C.c_void_p(out.data_ptr()), s))
    torch.cuda.synchronize()
    assert not out.any()


@pytest.mark.parametrize("pdename,lev,deg", [("continuity2", 4, 2), ("continuity3", 4, 3), ("continuity2", 3, 4)])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_rk3_step_equals_composed_step(dev, pdename, lev, deg, dtype):
    """One RK3 step with its sources formed inside it (for small-block plans one cooperative
    launch: three applies, two grid barriers) equals the step composed from three separate
    applies, the stage formulas of time_advance.m:177-204 and the sources summed on the host,
    to round-off."""
    import asgkron
    from asgkron import pdes
    from asgkron.steppers import RK3Stepper

    pde = getattr(pdes, pdename)(lev, 0.0)
    idx = asgkron.hash_table_sparse_nD(pde.levels, 8).idx1d()
    plan = asgkron.Plan.create(pde.term_mats(deg, construction_level=8), idx, deg)
    tdt = torch.float64 if dtype == "float64" else torch.float32
    st = RK3Stepper(plan, pde, idx, dtype=dtype)
    f0 = torch.from_numpy(np.random.default_rng(8).standard_normal(plan.dof)).to(dev, tdt)
    dt, t = pde.dt(0.01), 0.3
    x = f0.clone()
    st.step(x, t, dt)
    torch.cuda.synchronize()
    parts = [v.cpu().numpy() for v in st.vecs]
    s1, s2, s3 = [torch.from_numpy(sum((fn(tt) * v for fn, v in zip(st.tfac, parts)), np.zeros(plan.dof))).to(dev, tdt)
                  for tt in (t, t + 0.5 * dt, t + dt)]
    k1 = plan.apply(f0) + s1
    y = f0 + dt * 0.5 * k1
    k2 = plan.apply(y) + s2
    y = f0 + dt * (-k1 + 2 * k2)
    k3 = plan.apply(y) + s3
    want = f0 + dt * (k1 / 6 + 2 * k2 / 3 + k3 / 6)
    assert rel2(x.double().cpu().numpy(), want.double().cpu().numpy()) <= (1e-14 if dtype == "float64" else 1e-6)
    assert plan.device_status() == 0


@pytest.mark.parametrize("name,lev,deg,grid", [("continuity2_implicit_l2_d2", 2, 2, "SG"),
                                               ("continuity2_implicit_l4_d3", 4, 3, "SG"),
                                               ("continuity2_implicit_fg_l3_4_d3", [3, 4], 3, "FG")])
@pytest.mark.parametrize("mixed", ["matvec32", "inner32", "fp64"])
def test_backward_euler_matches_gold_trajectory(dev, name, lev, deg, grid, mixed):
    """5 backward-Euler steps at CFL 0.01 (source at t + dt) by GMRES + refinement on the GPU
    reproduce the reference's direct-solve gold trajectories."""
    import asgkron
    from asgkron import pdes
    from asgkron.steppers import be_step

    pde = pdes.continuity2(lev, 0.0)
    table = asgkron.hash_table_sparse_nD(pde.levels, 8, grid)
    idx = table.idx1d()
    plan = asgkron.Plan.create(pde.term_mats(deg, construction_level=8), idx, deg)
    f = torch.from_numpy(pde.initial_condition(deg, idx)).to(dev)
    dt = pde.dt(0.01)
    gold = np.load(os.path.join(G, "time_advance.npz"))
    for i in range(5):
        s = torch.from_numpy(pde.source_vector(deg, idx, (i + 1) * dt)).to(dev)
        f, info = be_step(plan, f, dt, source=s, mixed=mixed, tol=1e-13)
        torch.cuda.synchronize()
        assert info["converged"], (i, info)
        g = gold["%s_t%d" % (name, i)]
        assert rel2(f.cpu().numpy(), g) <= 1e-11, (i, info)


@pytest.mark.parametrize("name,lev,deg", [("continuity6_sg_l2_d3", 2, 3),
                                          ("continuity6_sg_l2_3_2_3_3_2_d2", [2, 3, 2, 3, 3, 2], 2)])
@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_rk3_continuity6_matches_gold_trajectory(dev, name, lev, deg, dtype):
    """continuity6 (the six-dimensional configuration's PDE, with its seven sources): 5 RK3
    steps on the GPU against gold/generated-inputs/time_advance (max_lev 4 for d > 3)."""
    import asgkron
    from asgkron import pdes
    from asgkron.steppers import RK3Stepper

    pde = pdes.continuity6(lev, 0.0)
    idx = asgkron.hash_table_sparse_nD(pde.levels, 4).idx1d()
    plan = asgkron.Plan.create(pde.term_mats(deg, construction_level=4), idx, deg)
    st = RK3Stepper(plan, pde, idx, dtype=dtype)
    tdt = torch.float64 if dtype == "float64" else torch.float32
    f = torch.from_numpy(pde.initial_condition(deg, idx)).to(dev, tdt)
    dt = pde.dt(0.01)
    gold = np.load(os.path.join(G, "time_advance.npz"))
    for i in range(5):
        st.step(f, i * dt, dt)
        torch.cuda.synchronize()
        g = gold["%s_t%d" % (name, i)]
        assert rel2(f.double().cpu().numpy(), g) <= (1e-13 if dtype == "float64" else 1e-6), i


@pytest.mark.parametrize("name,lev,deg,method", [("diffusion2_sg_l3_d3", 3, 3, "RK3"),
                                                 ("diffusion2_sg_l4_5_d2", [4, 5], 2, "RK3"),
                                                 ("diffusion2_implicit_sg_l4_d3", 4, 3, "BE"),
                                                 ("diffusion2_implicit_sg_l4_5_d2", [4, 5], 2, "BE")])
def test_diffusion2_matches_gold_trajectory(dev, name, lev, deg, method):
    """diffusion2.m with its Dirichlet data on the GPU: LDG operators, the boundary vector as
    rhs (RK3 stages on the device from its spatial parts; BE at t + dt), against the gold."""
    import asgkron
    from asgkron import pdes
    from asgkron.steppers import RK3Stepper, be_step

    pde = pdes.diffusion2(lev, case="reference")
    idx = asgkron.hash_table_sparse_nD(pde.levels, 8).idx1d()
    plan = asgkron.Plan.create(pde.term_mats(deg), idx, deg)
    f = torch.from_numpy(pde.initial_condition(deg, idx)).to(dev)
    dt = pde.dt(0.01)
    gold = np.load(os.path.join(G, "time_advance.npz"))
    st = RK3Stepper(plan, pde, idx) if method == "RK3" else None
    for i in range(5):
        if method == "RK3":
            st.step(f, i * dt, dt)
        else:
            bc = torch.from_numpy(pde.boundary_vector(deg, idx, (i + 1) * dt)).to(dev)
            f, info = be_step(plan, f, dt, source=bc, mixed=True, tol=1e-13)
            assert info["converged"], (i, info)
        torch.cuda.synchronize()
        g = gold["%s_t%d" % (name, i)]
        assert rel2(f.cpu().numpy(), g) <= 1e-11, i


@pytest.mark.parametrize("mixed", ["matvec32", "inner32", "fp64"])
def test_be_odd_block_size_vs_direct(dev, mixed):
    """deg 3 in 3-D (27-value blocks, so dof is not a multiple of 4): the Krylov basis vectors
    keep their 16-byte alignment; (I - dt A) x = b against a dense direct solve."""
    import asgkron
    from asgkron import pdes
    from asgkron.steppers import be_step

    pde = pdes.continuity3(3)
    idx = asgkron.hash_table_sparse_nD(pde.levels, 8).idx1d()
    mats = pde.term_mats(3)
    plan = asgkron.Plan.create(mats, idx, 3)
    assert plan.dof % 4 != 0
    f0 = np.random.default_rng(12).standard_normal(plan.dof)
    dt = 0.05
    _, A = O.apply_A_loop(mats, idx.astype(np.int64), 3, f0, build_A=True)
    want = O.backward_euler_step(A, f0, dt, np.zeros_like(f0))
    x, info = be_step(plan, torch.from_numpy(f0).to(dev), dt, mixed=mixed, tol=1e-12)
    torch.cuda.synchronize()
    assert info["converged"]
    assert rel2(x.cpu().numpy(), want) <= 1e-10


def test_rk3_cfg1_lf_upwind_vs_oracle(dev):
    """The CPU-runnable configuration: continuity2 lev 4 deg 2 (current PDE file, LF = -1),
    5 RK3 steps at CFL 0.01: GPU FP64 vs the oracle's RK3; FP32 within 1e-6."""
    import asgkron
    from asgkron import pdes
    from asgkron.steppers import RK3Stepper

    pde = pdes.continuity2(4)
    opde = O.continuity2(4)
    table = asgkron.hash_table_sparse_nD(pde.levels, 8)
    idx = table.idx1d()
    mats = pde.term_mats(2)
    plan = asgkron.Plan.create(mats, idx, 2)
    f0 = np.random.default_rng(0).standard_normal(plan.dof)
    dt = pde.dt(0.01)
    _, blocks = O.operator_two_scale(2, 8)
    idx64 = idx.astype(np.int64)
    omats = O.build_term_mats(opde, 2)
    fo = f0.copy()
    for i in range(5):
        fo = O.rk3_step(lambda v: O.apply_A_rows(omats, idx64, 2, v), fo, i * dt, dt,
                        lambda t: O.md_eval(opde, 2, opde.sources, idx64, blocks, t))
    for dtype, tol in (("float64", 1e-12), ("float32", 1e-6)):
        st = RK3Stepper(plan, pde, idx, dtype=dtype)
        f = torch.from_numpy(f0).to(dev, torch.float64 if dtype == "float64" else torch.float32)
        for i in range(5):
            st.step(f, i * dt, dt)
        torch.cuda.synchronize()
        assert rel2(f.double().cpu().numpy(), fo) <= tol, dtype


@pytest.mark.parametrize("mixed", ["matvec32", "inner32", "fp64"])
def test_be_solve_vs_direct(dev, mixed):
    """diffusion2 LDG (Dirichlet zero), lev 4 deg 3: (I - dt A) x = b by GMRES/IR vs a dense
    direct solve of the oracle-assembled A (the reference's AA \\ b, time_advance.m:349)."""
    import asgkron
    from asgkron import pdes
    from asgkron.steppers import be_step

    pde = pdes.diffusion2(4)
    table = asgkron.hash_table_sparse_nD(pde.levels, 8)
    idx = table.idx1d()
    mats = pde.term_mats(3)
    plan = asgkron.Plan.create(mats, idx, 3)
    f0 = pde.initial_condition(3, idx) + 1e-3 * np.random.default_rng(2).standard_normal(plan.dof)
    dt = pde.dt(1.0)
    _, A = O.apply_A_loop(mats, idx.astype(np.int64), 3, f0, build_A=True)
    want = O.backward_euler_step(A, f0, dt, np.zeros_like(f0))
    x, info = be_step(plan, torch.from_numpy(f0).to(dev), dt, mixed=mixed, tol=1e-10)
    assert info["converged"] and info["rel_residual"] <= 1e-10, info
    assert rel2(x.cpu().numpy(), want) <= 1e-9


def test_be_cfg3_ten_steps_mixed_vs_fp64(dev):
    """Implicit configuration: diffusion2 SG lev 8, deg 4 (20,480 DOF), dt = h^2, 10 steps from
    sin(pi x) sin(pi y) + 1e-3 N(0,1) (seed 2): GMRES(30) with the FP32 operator (FP64 Arnoldi)
    and FP64 GMRES(30) both reach 1e-10 relative residual each step and agree."""
    import asgkron
    from asgkron import pdes
    from asgkron.steppers import be_step

    pde = pdes.diffusion2(8)
    table = asgkron.hash_table_sparse_nD(pde.levels, 8)
    idx = table.idx1d()
    mats = pde.term_mats(4)
    plan = asgkron.Plan.create(mats, idx, 4)
    f0 = pde.initial_condition(4, idx) + 1e-3 * np.random.default_rng(2).standard_normal(plan.dof)
    dt = pde.dt(1.0)
    fm = torch.from_numpy(f0).to(dev)
    fd = fm.clone()
    for step in range(10):
        fm, im = be_step(plan, fm, dt, mixed=True)
        fd, idd = be_step(plan, fd, dt, mixed=False)
        assert im["converged"] and im["rel_residual"] <= 1e-10, (step, im)
        assert idd["converged"] and idd["rel_residual"] <= 1e-10, (step, idd)
    assert rel2(fm.cpu().numpy(), fd.cpu().numpy()) <= 1e-9


@pytest.mark.parametrize("lev,deg,mixed", [(4, 2, "matvec32"), (4, 2, "inner32"), (4, 3, "fp64"), (6, 4, "matvec32"),
                                            (6, 4, "inner32"), (6, 4, "fp64")])
def test_be_fused_cycle_vs_per_phase_cycle(dev, lev, deg, mixed):
    """Plans on the small-block kernel run each GMRES cycle as one cooperative launch; the same
    plan switched to the warp-chain kernel runs the kernel-per-phase cycle.  Both solve
    (I - dt A) x = b to the same tolerance and agree with each other."""
    import asgkron
    from asgkron import pdes
    from asgkron._lib import KERNEL_CHAIN_WARP, KERNEL_NAMES
    from asgkron.steppers import be_step

    pde = pdes.diffusion2(lev)
    idx = asgkron.hash_table_sparse_nD(pde.levels, 8).idx1d()
    plan = asgkron.Plan.create(pde.term_mats(deg), idx, deg)
    assert KERNEL_NAMES[plan.stats()["kernel_kind"]] == "single_mode_small"
    f0 = pde.initial_condition(deg, idx) + 1e-3 * np.random.default_rng(5).standard_normal(plan.dof)
    dt = pde.dt(1.0)
    f = torch.from_numpy(f0).to(dev)
    xf, inf_f = be_step(plan, f, dt, mixed=mixed, tol=1e-11, restart=20)
    xf2, _ = be_step(plan, f, dt, mixed=mixed, tol=1e-11, restart=20)
    plan.set_kernel(KERNEL_CHAIN_WARP)
    xp, inf_p = be_step(plan, f, dt, mixed=mixed, tol=1e-11, restart=20)
    torch.cuda.synchronize()
    assert inf_f["converged"] and inf_p["converged"], (inf_f, inf_p)
    assert inf_f["rel_residual"] <= 1e-11 and inf_p["rel_residual"] <= 1e-11
    assert torch.equal(xf, xf2)  # fixed-order reductions: the fused cycle is reproducible
    assert rel2(xf.cpu().numpy(), xp.cpu().numpy()) <= 1e-9


def test_be_fused_barrier_timeout_reports_and_recovers(dev):
    """The one-launch solve's grid barriers wait a bounded time.  With CTA 0 withholding one
    arrival (the test hook), every CTA's wait runs out (~1 s), the solve returns
    ASG_ERR_TIMEOUT, and the context stays usable: the same solve then succeeds and matches
    a direct solve."""
    import asgkron
    from asgkron import pdes
    from asgkron._lib import AsgError, check, lib
    from asgkron.steppers import be_step

    pde = pdes.diffusion2(4)
    idx = asgkron.hash_table_sparse_nD(pde.levels, 8).idx1d()
    mats = pde.term_mats(2)
    plan = asgkron.Plan.create(mats, idx, 2)
    f0 = pde.initial_condition(2, idx) + 1e-3 * np.random.default_rng(7).standard_normal(plan.dof)
    dt = pde.dt(1.0)
    f = torch.from_numpy(f0).to(dev)
    for mixed in (True, False):
        check(lib().asg_debug_withhold_arrival(5))
        with pytest.raises(AsgError, match="grid barrier"):
            be_step(plan, f, dt, mixed=mixed)
    x, info = be_step(plan, f, dt, mixed=True, tol=1e-11)
    torch.cuda.synchronize()
    assert info["converged"]
    _, A = O.apply_A_loop(mats, idx.astype(np.int64), 2, f0, build_A=True)
    want = O.backward_euler_step(A, f0, dt, np.zeros_like(f0))
    assert rel2(x.cpu().numpy(), want) <= 1e-9


@pytest.mark.parametrize("name,lev,deg", [("diffusion2", 4, 3), ("continuity2", 4, 2), ("continuity3", 3, 2)])
def test_assemble_bsr_matches_oracle(dev, name, lev, deg):
    """The assembled operator (apply_A.m's build_A branch, apply_A.m:170-180,246-248) on the
    GPU: the reference work model equals the oracle's dense A; the structured model equals it
    to the dropped magnitudes and its product with f equals the apply."""
    import asgkron

    from cases import problem

    pde, table, idx, mats = problem(name, lev, deg)
    f = np.random.default_rng(7).standard_normal(idx.shape[0] * deg ** idx.shape[1])
    _, Aref = O.apply_A_loop(mats, idx.astype(np.int64), deg, f, build_A=True)
    full = asgkron.Plan.create(mats, idx, deg, structure="none")
    A_none = full.assemble_bsr().toarray()
    assert rel2(A_none, Aref) <= 1e-14
    plan = asgkron.Plan.create(mats, idx, deg)
    A = plan.assemble_bsr()
    assert rel2(A.toarray(), Aref) <= 1e-12
    y = plan.apply(torch.from_numpy(f).to(dev))
    torch.cuda.synchronize()
    assert rel2(A @ f, y.cpu().numpy()) <= 1e-13
    full.close()
    plan.close()


def test_be_cfg3_against_direct_solve(dev):
    """Implicit configuration (diffusion2 SG lev 8, deg 4, 20,480 DOF, dt = h^2, ten steps from
    sin(pi x) sin(pi y) + 1e-3 N(0,1), seed 2).  The reference assembles A and solves
    (I - dt A) f1 = b directly (time_advance.m:333-349): here A is assembled on the GPU as
    block-sparse rows and factored once by scipy's sparse LU on the host, the checker.  GMRES(30)
    with iterative refinement in each precision mode -- the FP32 operator inside FP64 Arnoldi
    (the configuration's mode), the FP32 inner cycle, and FP64 -- reaches 1e-10 relative
    residual every step, and its trajectory matches the direct one to 1e-9."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as sla

    import asgkron
    from asgkron import pdes
    from asgkron.steppers import be_step

    pde = pdes.diffusion2(8)
    idx = asgkron.hash_table_sparse_nD(pde.levels, 8).idx1d()
    plan = asgkron.Plan.create(pde.term_mats(4), idx, 4)
    assert plan.dof == 20480
    f0 = pde.initial_condition(4, idx) + 1e-3 * np.random.default_rng(2).standard_normal(plan.dof)
    dt = pde.dt(1.0)
    A = plan.assemble_bsr().tocsc()
    M = (sp.identity(plan.dof, format="csc") - dt * A).tocsc()
    lu = sla.splu(M, permc_spec="MMD_AT_PLUS_A")
    direct = [f0]
    for _ in range(10):
        direct.append(lu.solve(direct[-1]))
    for k in range(1, 11):  # the direct solve itself
        assert np.linalg.norm(M @ direct[k] - direct[k - 1]) <= 1e-12 * np.linalg.norm(direct[k - 1])
    for mode in ("matvec32", "inner32", "fp64"):
        f = torch.from_numpy(f0).to(dev)
        for step in range(10):
            f, info = be_step(plan, f, dt, mixed=mode)
            assert info["converged"] and info["rel_residual"] <= 1e-10, (mode, step, info)
        torch.cuda.synchronize()
        got = f.cpu().numpy()
        assert rel2(got, direct[10]) <= 1e-9, mode
        # the last step's residual against the assembled matrix, from the GPU's own previous state
    plan.close()
