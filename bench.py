#!/usr/bin/env python
"""Benchmark: apply_A throughput (GDOF/s) on one GB300, FP32 vs FP64.

Workload (default): continuity6, SG level 4, degree 4 -- 501 elements of 4^6 = 4096 values,
2,052,096 DOF, six terms each a DG d/dx_k in one dimension and the mass (identity) in the
others; f ~ N(0,1) FP32 seed 4 (synthetic: the reference ships no dataset for this path).
One step = one y = A*f over the whole element set.  Inputs are 8.2 MB (FP32), smaller than
the 129 MB L2, so L2 is flushed (512 MB device write) before every timed step, outside the
timed apply.

Output: one JSON line (rank 0).  ``value`` is device-resident throughput of the FP32
structured kernel; ``e2e`` is the same metric through the host-pointer C ABI call
(asg_apply_host_f32: H2D of f from pinned memory, apply, synchronise; y is pinned, so the
kernel stores it over the host link as rows finish instead of a D2H copy after the apply);
``roofline`` uses the compulsory-bytes model of the path; ``cpu_baseline`` times the C
restatement of the reference loop on a bounded row sample on the host cores.
``--impl reference`` times that CPU implementation alone (the reference is MATLAB and
cannot run on the box; the faithful C port stands in for it).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "dg-sparsegrid_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "apply_A GDOF/s & % roofline: FP32 vs FP64 on-GPU at <=1e-6 rel err"
UNIT = "GDOF/s"
WORKLOAD = "continuity6 SG lev4 deg4 (501 elements x 4096 DOF, 6 terms, all pairs)"
DATA = "synthetic (continuity6 operators from the DG builder; f ~ N(0,1) seed 4)"
L2_NOTE = "inputs (8.2 MB) below L2: L2 flushed (512 MB device write) before every timed GPU step"


def workload_config(dof):
    """The ``config`` both arms print (identical: the workload, not the implementation)."""
    return {"workload": WORKLOAD, "dof": dof, "l2": L2_NOTE}
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ref-budget", type=float, default=150.0,
                    help="reference arm: seconds of host work for warmup + steps (sets the rows per step)")
    ap.add_argument("--skip-variants", action="store_true")
    ap.add_argument("--sharded", action="store_true",
                    help="run the row-slice (multi-GPU) path even on one GPU: one slice holding every row")
    ap.add_argument("--replicas", action="store_true",
                    help="with several GPUs: run independent copies of the one-GPU workload (weak scaling) instead "
                         "of splitting its rows across the GPUs")
    ap.add_argument("--workload", default="continuity6", choices=["continuity6", "batched", "implicit"],
                    help="batched: the 256-problem persistent-launch configuration; implicit: the "
                         "backward-Euler diffusion2 configuration (each its own JSON line)")
    ap.add_argument("--batch-problems", type=int, default=256,
                    help="batched workload: number of problems drawn (the configuration has 256)")
    ap.add_argument("--batch-max-level", type=int, default=7,
                    help="batched workload: highest SG level drawn (the configuration has 7)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def build_workload():
    import asgkron
    from asgkron import pdes

    pde = pdes.continuity6(4)
    deg = 4
    table = asgkron.hash_table_sparse_nD(pde.levels, 4)
    idx = table.idx1d()
    mats = pde.term_mats(deg)
    return pde, deg, idx, mats


def algorithmic_bytes(s, dof, T, d, n1d, N, pairs):
    """Compulsory bytes per apply: read f, write y, read the operators, read the pair list."""
    return s * (2 * dof + T * d * n1d * n1d) + 4 * (N + 1 + pairs)


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.path = tempfile.mktemp(prefix="clocks_", suffix=".csv")
        self.proc = None
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.QUERY, "--format=csv,noheader,nounits",
                                          "-i", str(gpu_index), "-lms", "100"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        self.t_start = time.time()

    def stop(self, t0, t1):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        rows = []
        with open(self.path) as fh:
            for line in fh:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        # nvidia-smi -lms writes one line per period from t_start; keep the ones in [t0, t1]
        n = len(rows)
        if n == 0:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        period = 0.1
        sel = [r for k, r in enumerate(rows) if t0 - period <= self.t_start + k * period <= t1 + period]
        note = []
        if not sel:
            sel = rows
            note.append("timed region shorter than the sampling period; samples around it")

        def num(v):
            try:
                return float(v)
            except ValueError:
                return None

        sm = [num(r[1]) for r in sel if num(r[1]) is not None]
        mx = [num(r[2]) for r in sel if num(r[2]) is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in sel for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons + note, "samples": len(sel)}


def oracle_workload():
    """The continuity6 workload (SG level 4, degree 4) built by the oracle alone: element table,
    1-D indices and operators from the CPU restatement, no product code loaded."""
    from oracle import asgard_oracle as O

    pde = O.continuity6(4)
    mats = O.build_term_mats(pde, 4)
    levels, cells, _ = O.hash_table_sparse_nd([4] * 6, 4)
    return mats, O.element_idx1d(levels, cells), 4


def time_reference_rows(mats, idx, deg, f64, rows, cores):
    """Seconds for the reference loop (oracle/apply_a_ref.c: every one of the N columns x 6
    terms x the 6-mode chain) over the given whole rows, on ``cores`` threads."""
    from oracle import cref

    t0 = time.perf_counter()
    cref.apply_rows(mats, idx, deg, f64, rows=rows, nthreads=cores)
    return time.perf_counter() - t0


def cpu_baseline(f64, budget_s=12.0):
    """The reference loop on the host cores over whole rows (all N columns each), as many rows
    as fit in about ``budget_s`` seconds (the whole element set when it fits)."""
    import numpy as np

    mats, idx, deg = oracle_workload()
    N = idx.shape[0]
    B = deg ** idx.shape[1]
    cores = os.cpu_count() or 1
    probe = np.arange(0, N, max(1, N // cores))[:cores].astype(np.int32)
    time_reference_rows(mats, idx, deg, f64, probe[:2], cores)  # build, page-in
    per_row = time_reference_rows(mats, idx, deg, f64, probe, cores) / probe.size
    nrows = int(min(N, max(cores, budget_s / per_row)))
    rows = np.linspace(0, N - 1, nrows).astype(np.int32)
    dt = time_reference_rows(mats, idx, deg, f64, rows, cores)
    return {"value": nrows * B / dt / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%s: %d of %d whole rows (each over all %d columns x 6 terms x the 6-mode chain), FP64, "
                      "%.2f s" % ("the whole element set" if nrows == N else "a row sample", nrows, N, N, dt)}


def run_reference(args, rank):
    """Time the CPU implementation of the path on the host cores: the C restatement of the
    reference loop (apply_A.m:102-236, all pairs, 6 terms, 6-mode chain, FP64, OpenMP over
    rows).  Operators, element table and f come from the oracle alone (no product code).  A
    step is one y = A f over the whole element set when warmup + steps fit in about
    ``--ref-budget`` seconds, otherwise the same number of whole rows in every step (stated in
    ``sample``)."""
    import numpy as np

    if rank != 0:
        return
    mats, idx, deg = oracle_workload()
    N = idx.shape[0]
    B = deg ** idx.shape[1]
    f64 = np.random.default_rng(4).standard_normal(N * B)
    cores = os.cpu_count() or 1
    probe = np.arange(0, N, max(1, N // cores))[:cores].astype(np.int32)
    time_reference_rows(mats, idx, deg, f64, probe[:2], cores)  # build, page-in
    per_row = time_reference_rows(mats, idx, deg, f64, probe, cores) / probe.size
    steps = max(1, args.steps)
    total = steps + max(args.warmup, 0)
    nrows = int(min(N, max(cores, args.ref_budget / total / per_row)))
    rows = np.linspace(0, N - 1, nrows).astype(np.int32)
    for _ in range(max(args.warmup, 0)):
        time_reference_rows(mats, idx, deg, f64, rows, cores)
    t_all = 0.0
    for _ in range(steps):
        t_all += time_reference_rows(mats, idx, deg, f64, rows, cores)
    per_step = t_all / steps
    value = nrows * B / per_step / 1e9
    sample = ("the whole element set, %d rows x %d columns x 6 terms x the 6-mode chain, FP64" % (N, N) if nrows == N
              else "%d of %d whole rows per step (each over all %d columns x 6 terms x the 6-mode chain), FP64"
                   % (nrows, N, N))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus, "steps": steps,
        "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": DATA,
        "config": workload_config(N * B),
        "sample": sample,
        "implementation": "C restatement of apply_A.m's loop (oracle/apply_a_ref.c), OpenMP over rows on %d host "
                          "threads; operators and element table from the oracle (the MATLAB reference cannot run "
                          "on the box)" % cores,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "product_code_loaded": "asgkron" in sys.modules,
    }
    print(json.dumps(line), flush=True)


def time_device(plan, f, y, flush, steps, warmup, stream):
    import torch

    for _ in range(warmup):
        flush()
        plan.apply(f, y, stream)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for s, e in ev:
        flush()
        s.record(stream)
        plan.apply(f, y, stream)
        e.record(stream)
    torch.cuda.synchronize()
    return [s.elapsed_time(e) for s, e in ev]


def forward_backward(plan, f, ystar, flush, steps, stream, dof, n1d):
    """Differentiation step on continuity6 (FP32): r = A f - y* (the residual apply: the
    subtraction made in the apply's own stores), fbar = A^T r and the gradients of
    L = 1/2 ||A f - y*||^2 with respect to the applied 1-D operators.  Three launches per step
    (residual apply, adjoint, operator gradient), timed as one region."""
    import ctypes as C

    import torch
    from asgkron._lib import check, lib

    T, D = plan.T, plan.D
    active = plan.active_factors()
    ptrs, lds, keep = (C.c_void_p * (T * D))(), (C.c_int * (T * D))(), []
    n_active = 0
    for t in range(T):
        for d in range(D):
            if active[t][d]:
                n = plan.term_mats[t][d].shape[0]
                g = torch.zeros(n * n, dtype=f.dtype, device=f.device)
                keep.append(g)
                ptrs[t * D + d], lds[t * D + d] = g.data_ptr(), n
                n_active += 1
    r, fbar = torch.empty_like(f), torch.empty_like(f)
    sp = C.c_void_p(stream.cuda_stream)

    def step():
        plan.apply_residual(f, ystar, r, stream)
        plan.apply_T(r, fbar, stream)
        check(lib().asg_grad_ops_f32(plan.handle, C.c_void_p(f.data_ptr()), C.c_void_p(r.data_ptr()), ptrs, lds, sp))

    for _ in range(3):
        flush()
        step()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for s, e in ev:
        flush()
        s.record(stream)
        step()
        e.record(stream)
    torch.cuda.synchronize()
    ms = sum(s.elapsed_time(e) for s, e in ev) / steps
    st = plan.stats()
    # compulsory bytes: forward and adjoint as the forward model, plus y* read by the residual
    # apply; the gradient reads f and r and writes the applied operators' gradients
    fwd = algorithmic_bytes(4, dof, T, D, n1d, plan.N, st["num_pairs"])
    alg = 2 * fwd + 4 * dof + 4 * (2 * dof + n_active * n1d * n1d)
    return {"value": dof / (ms * 1e-3) / 1e9, "ms": ms, "launches_per_step": 3,
            "algorithmic_bytes": alg, "achieved_gbs": alg / (ms * 1e-3) / 1e9}


def implicit_steps(dev, nsteps=10):
    """Implicit configuration: diffusion2 LDG (Dirichlet zero), SG level 8, degree 4 (20,480
    DOF), dt = h^2 (CFL 1), f0 = projection of sin(pi x) sin(pi y) + 1e-3 N(0,1) (seed 2); ten
    backward-Euler steps by GMRES(30) + iterative refinement to 1e-10 relative residual, once
    with the FP32 matvec inside (mixed) and once all FP64.  Host-driven solver: wall-clock."""
    import numpy as np
    import torch

    import asgkron
    from asgkron import pdes
    from asgkron.steppers import be_step

    pde = pdes.diffusion2(8)
    idx = asgkron.hash_table_sparse_nD(pde.levels, 8).idx1d()
    plan = asgkron.Plan.create(pde.term_mats(4), idx, 4)
    f0 = pde.initial_condition(4, idx) + 1e-3 * np.random.default_rng(2).standard_normal(plan.dof)
    dt = pde.dt(1.0)
    out = {}
    finals = {}
    # matvec32: FP32 operator inside FP64 Arnoldi (dot products, norms, updates): the
    # configuration's mixed mode; inner32: the whole inner cycle in FP32; fp64: everything FP64
    # each mode runs the ten steps twice from f0 (identical work, bitwise identical results);
    # the faster pass is reported, so one host-side stall does not stand for the mode
    for mode, mixed in (("mixed", "matvec32"), ("mixed_fp32_inner", "inner32"), ("fp64", "fp64")):
        be_step(plan, torch.from_numpy(f0).to(dev), dt, mixed=mixed)  # warm-up (workspace, first launches)
        passes = []
        for _ in range(2):
            f = torch.from_numpy(f0).to(dev)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            outer = inner = 0
            worst = 0.0
            for _ in range(nsteps):
                f, info = be_step(plan, f, dt, mixed=mixed)
                outer += info["outer_iters"]
                inner += info["inner_iters"]
                worst = max(worst, info["rel_residual"])
            torch.cuda.synchronize()
            passes.append((time.perf_counter() - t0) / nsteps * 1e3)
        out[mode] = {"ms_per_step": min(passes), "passes_ms_per_step": passes, "outer_iters": outer,
                     "inner_iters": inner, "max_rel_residual": worst}
        finals[mode] = f
    out["mixed_speedup"] = out["fp64"]["ms_per_step"] / out["mixed"]["ms_per_step"]
    out["mixed_fp32_inner_speedup"] = out["fp64"]["ms_per_step"] / out["mixed_fp32_inner"]["ms_per_step"]
    out["modes"] = {"mixed": "FP32 operator, FP64 basis / Arnoldi dot products and norms / Givens / update",
                    "mixed_fp32_inner": "the whole inner GMRES cycle in FP32", "fp64": "all FP64"}
    # the operator application alone, both precisions (L2-resident, as inside the solver)
    stream = torch.cuda.current_stream(dev)
    x64 = torch.from_numpy(f0).to(dev)
    for name, x in (("apply_fp64_us", x64), ("apply_fp32_us", x64.float())):
        ms = time_device(plan, x, torch.empty_like(x), lambda: None, 200, 10, stream)
        out[name] = 1e3 * sum(ms) / len(ms)
    out["rel_diff_mixed_vs_fp64"] = float(torch.linalg.norm(finals["mixed"] - finals["fp64"]) /
                                          torch.linalg.norm(finals["fp64"]))
    out["rel_diff_mixed_fp32_inner_vs_fp64"] = float(torch.linalg.norm(finals["mixed_fp32_inner"] - finals["fp64"]) /
                                                     torch.linalg.norm(finals["fp64"]))
    out["dof"] = plan.dof
    plan.close()
    return out


def adaptive_plan_updates(dev, nsteps=5):
    """Plan maintenance under adaptivity: the continuity2 adaptive run (SG level 3, degree 4,
    central flux, relative threshold 1e-3, RK3 at CFL 0.01: the setup of the reference's
    continuity2_ad_sg_l3_d4 gold run, 20 -> 112 elements), every step on the GPU (FP64 RK3).
    Each adapted table needs a plan: "rebuild" creates one from the table's rechained operators
    (asg_plan_create); "update" keeps one plan made from the maximum-level operators and swaps
    its table in place (asg_plan_update_elements).  Reports host milliseconds per plan change
    (synchronised) and the difference of the final states."""
    import numpy as np
    import torch

    import asgkron
    from asgkron import pdes
    from asgkron.adapt import AdaptiveRun, operator_extent, update_plan
    from asgkron.steppers import RK3Stepper

    out = {}
    finals = {}
    for mode in ("rebuild", "update"):
        pde = pdes.continuity2(3, 0.0)
        run = AdaptiveRun(pde, 4, asgkron.hash_table_sparse_nD([3, 3], 8), 1e-3)
        dt = pdes.continuity2(3, 0.0).dt(0.01)
        st = {"plan": None, "ms": [], "tables": 0}

        def step(r, fv, t):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if mode == "rebuild":
                if st["plan"] is not None:
                    st["plan"].close()
                st["plan"] = asgkron.Plan.create(r.term_mats(), r.idx1d, 4)
            elif st["plan"] is None:
                top = r.pde.rechain_term_mats(4, [8, 8], 8, r._pterms)
                st["plan"] = asgkron.Plan.create(top, r.idx1d, 4, op_blocks=operator_extent(top, 4))
            else:
                st["plan"] = update_plan(st["plan"], r.table, term_mats=r.term_mats())
            torch.cuda.synchronize()
            st["ms"].append((time.perf_counter() - t0) * 1e3)
            st["tables"] += 1
            x = torch.from_numpy(np.ascontiguousarray(fv)).to(dev)
            RK3Stepper(st["plan"], pde, r.idx1d).step(x, t, dt)
            return x.cpu().numpy()

        f = run.initial()
        for i in range(nsteps):
            f = run.advance(f, i * dt, step)
        finals[mode] = f
        ms = st["ms"]
        out[mode] = {"plan_changes": st["tables"], "first_ms": ms[0],
                     "mean_ms_after_first": sum(ms[1:]) / max(1, len(ms) - 1), "elements_final": run.table.num_elems}
        st["plan"].close()
    out["speedup_after_first"] = out["rebuild"]["mean_ms_after_first"] / out["update"]["mean_ms_after_first"]
    out["final_state_rel_diff"] = float(np.linalg.norm(finals["rebuild"] - finals["update"]) /
                                        np.linalg.norm(finals["rebuild"]))
    return out


def precision_continuity3(dev, flush, stream):
    """Precision configuration: continuity3 SG level 6, degree 3 (18,576 DOF), f ~ N(0,1)
    seed 1: FP64 and FP32 applies, FP32 relative 2-norm error against FP64."""
    import numpy as np
    import torch

    import asgkron
    from asgkron import pdes

    pde = pdes.continuity3(6)
    idx = asgkron.hash_table_sparse_nD(pde.levels, 8).idx1d()
    plan = asgkron.Plan.create(pde.term_mats(3), idx, 3)
    f64 = torch.from_numpy(np.random.default_rng(1).standard_normal(plan.dof)).to(dev)
    f32 = f64.float()
    y64, y32 = torch.empty_like(f64), torch.empty_like(f32)
    m64 = time_device(plan, f64, y64, flush, 100, 5, stream)
    m32 = time_device(plan, f32, y32, flush, 100, 5, stream)
    err = float(torch.linalg.norm(y32.double() - y64) / torch.linalg.norm(y64))
    t64, t32 = sum(m64) / len(m64), sum(m32) / len(m32)
    out = {"dof": plan.dof, "fp64": {"value": plan.dof / (t64 * 1e-3) / 1e9, "ms": t64},
           "fp32": {"value": plan.dof / (t32 * 1e-3) / 1e9, "ms": t32}, "fp32_rel_err_vs_fp64": err,
           "kernel": asgkron._lib.KERNEL_NAMES[plan.stats()["kernel_kind"]]}
    plan.close()
    return out


def batched_measure(dev, count, max_level, steps, warmup):
    """Batching configuration: ``count`` independent problems, each d ~ U{2,3,4}, SG level ~
    U{3..max_level}, degree ~ U{2..4} (seed 3), d terms of dense N(0, 1/deg) 1-D operators (no
    structure, so every (pair, term) of all N^2 pairs is executed: the reference work model),
    f ~ N(0,1).  One step = one persistent launch over all problems (FP32, tuned, replayed from
    a CUDA graph).  Baseline: the same problems as sequential FP64 single-problem launches.  The
    256-problem draw's inputs (62 MB of f, 5.8 GB of work lists at 4 bytes per work entry)
    exceed L2, so no flush is needed.  Returns the measurements (dict)."""
    import numpy as np
    import torch

    import asgkron
    from asgkron.batch import Batch

    rng = np.random.default_rng(3)
    plans, f64s = [], []
    flops, wl_bytes = 0.0, 0
    t_build = time.perf_counter()
    for _ in range(count):
        d = int(rng.choice([2, 3, 4]))
        lev = int(rng.integers(3, max_level + 1))
        deg = int(rng.integers(2, 5))
        idx = asgkron.hash_table_sparse_nD([lev] * d, 8).idx1d()
        n = deg * 2 ** lev
        mats = [[rng.normal(0.0, 1.0 / np.sqrt(deg), (n, n)) for _ in range(d)] for _ in range(d)]
        p = asgkron.Plan.create(mats, idx, deg, structure="none")
        p.term_mats = None  # the plan holds its own packed copy; drop the host operators
        st = p.stats()
        flops += st["flops_executed"]
        wl_bytes += 4 * st["num_entries"]  # one 4-byte (column, term) word per work entry
        plans.append(p)
        f64s.append(torch.from_numpy(rng.standard_normal(p.dof)).to(dev))
    build_s = time.perf_counter() - t_build
    dof = sum(p.dof for p in plans)
    f32s = [f.float() for f in f64s]
    y32s = [torch.empty_like(f) for f in f32s]
    y64s = [torch.empty_like(f) for f in f64s]
    b = Batch(plans)
    b.set_io(f32s, y32s)
    b.tune()
    g = b.capture()
    stream = torch.cuda.current_stream(dev)
    for _ in range(max(3, warmup)):
        g.replay()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for s, e in ev:
        s.record(stream)
        g.replay()
        e.record(stream)
    torch.cuda.synchronize()
    ms = sum(s.elapsed_time(e) for s, e in ev) / steps
    # baseline: the same problems one FP64 launch after another
    for p, f, y in zip(plans, f64s, y64s):
        p.apply(f, y, stream)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record(stream)
    for p, f, y in zip(plans, f64s, y64s):
        p.apply(f, y, stream)
    e.record(stream)
    torch.cuda.synchronize()
    ms64 = s.elapsed_time(e)
    errs = [float(torch.linalg.norm(a.double() - c) / torch.linalg.norm(c)) for a, c in zip(y32s, y64s)]
    # end to end: pinned host f in, one batched launch, y back
    fh = [f.cpu().pin_memory() for f in f32s]
    yh = [torch.empty_like(t).pin_memory() for t in fh]
    e2e_steps = max(1, min(steps, 5))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        for h, d_ in zip(fh, f32s):
            d_.copy_(h, non_blocking=True)
        g.replay()
        for h, d_ in zip(yh, y32s):
            h.copy_(d_, non_blocking=True)
        torch.cuda.synchronize()
    e2e_ms = (time.perf_counter() - t0) / e2e_steps * 1e3
    out = {"problems": count, "max_level": max_level, "dof": dof, "ms": ms, "value": dof / (ms * 1e-3) / 1e9,
           "gflops_per_s": flops / (ms * 1e-3) / 1e9, "flops_per_step": flops, "work_list_bytes": wl_bytes,
           "tuned": b.info(), "build_s": build_s,
           "fp64_sequential_launches": {"ms": ms64, "value": dof / (ms64 * 1e-3) / 1e9,
                                        "gflops_per_s": flops / (ms64 * 1e-3) / 1e9},
           "speedup_vs_fp64_sequential": ms64 / ms,
           "fp32_rel_err_vs_fp64": {"max": max(errs), "median": statistics.median(errs)},
           "e2e_ms": e2e_ms, "e2e_value": dof / (e2e_ms * 1e-3) / 1e9}
    b.close()
    for p in plans:
        p.close()
    return out


def run_batched(args, rank, local):
    """The batching configuration alone (rank 0): see batched_measure; one JSON line."""
    import torch

    if rank != 0:
        return
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    steps = max(1, min(args.steps, 20))
    r = batched_measure(dev, args.batch_problems, args.batch_max_level, steps, args.warmup)
    wl = r["work_list_bytes"]
    line = {
        "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": max(3, args.warmup), "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (dense N(0,1/deg) operators, f ~ N(0,1), seed 3)",
        "config": {"workload": "batched: %d problems, d in {2,3,4}, SG lev 3..%d, deg 2..4, all pairs"
                               % (args.batch_problems, args.batch_max_level),
                   "dof": r["dof"], "flops_per_step": r["flops_per_step"],
                   "l2": ("inputs larger than L2 (%.3g GB work lists)" if wl > 129e6 else
                          "work lists within L2 (%.3g GB), no flush") % (wl / 1e9),
                   "launch": "one persistent launch replayed from a CUDA graph", "tuned": r["tuned"]},
        "compute": {"gflops_per_s": r["gflops_per_s"]},
        "variants": {"fp64_sequential_launches": dict(r["fp64_sequential_launches"], count=args.batch_problems),
                     "speedup_vs_fp64_sequential": r["speedup_vs_fp64_sequential"],
                     "fp32_rel_err_vs_fp64": r["fp32_rel_err_vs_fp64"]},
        "e2e": {"value": r["e2e_value"], "unit": UNIT, "h2d_bytes_per_step": 4 * r["dof"],
                "d2h_bytes_per_step": 4 * r["dof"], "ms_per_step": r["e2e_ms"]},
        "gpu_launches": steps * 2,  # counter reset (memset node) + the persistent kernel per replay
    }
    print(json.dumps(line), flush=True)


def batch_draws(count, max_level, seed=3):
    """The batched generator's problems as (d, lev, deg, N), with every operator and f drawn
    and discarded so that the random stream advances exactly as in run_batched."""
    import numpy as np

    import asgkron

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        d = int(rng.choice([2, 3, 4]))
        lev = int(rng.integers(3, max_level + 1))
        deg = int(rng.integers(2, 5))
        N = asgkron.hash_table_sparse_nD([lev] * d, 8).idx1d().shape[0]
        n = deg * 2 ** lev
        for _ in range(d * d):
            rng.normal(0.0, 1.0 / np.sqrt(deg), (n, n))
        rng.standard_normal(N * deg ** d)
        out.append((d, lev, deg, N))
    return out


def batch_costs(draws):
    """Reference-model flops of each problem: all N^2 pairs x d terms x d factors x 2 deg^(d+1)."""
    return [float(N) * N * d * d * 2.0 * deg ** (d + 1) for d, lev, deg, N in draws]


def run_batched_sharded(args, rank, world, local):
    """The batched configuration on ``world`` GPUs: the problems are split by cost
    (asgkron.batch.partition_problems, no communication on the data path); each rank builds
    its own problems (the same draws as run_batched), tunes and captures its batch, and
    replays it.  value = all ranks' DOF / the slowest rank's time per replay (strong scaling:
    the 256 problems are fixed)."""
    import numpy as np
    import torch
    import torch.distributed as dist

    import asgkron
    from asgkron.batch import Batch, partition_problems

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    dist.init_process_group("nccl", device_id=dev)
    try:
        draws = batch_draws(args.batch_problems, args.batch_max_level)
        mine = set(partition_problems(batch_costs(draws), world)[rank])
        rng = np.random.default_rng(3)
        plans, f32s = [], []
        flops = 0.0
        for k in range(args.batch_problems):  # the draws of run_batched, in its order
            d = int(rng.choice([2, 3, 4]))
            lev = int(rng.integers(3, args.batch_max_level + 1))
            deg = int(rng.integers(2, 5))
            idx = asgkron.hash_table_sparse_nD([lev] * d, 8).idx1d()
            n = deg * 2 ** lev
            mats = [[rng.normal(0.0, 1.0 / np.sqrt(deg), (n, n)) for _ in range(d)] for _ in range(d)]
            f = rng.standard_normal(idx.shape[0] * deg ** d)
            if k not in mine:
                continue
            p = asgkron.Plan.create(mats, idx, deg, structure="none")
            p.term_mats = None
            flops += p.stats()["flops_executed"]
            plans.append(p)
            f32s.append(torch.from_numpy(f).to(dev).float())
        steps = max(1, min(args.steps, 20))
        stream = torch.cuda.current_stream(dev)
        ms = e2e_ms = 0.0
        info = {}
        if plans:
            y32s = [torch.empty_like(f) for f in f32s]
            b = Batch(plans)
            b.set_io(f32s, y32s)
            b.tune()
            g = b.capture()
            info = b.info()
            for _ in range(max(3, args.warmup)):
                g.replay()
        torch.cuda.synchronize()
        dist.barrier()
        if plans:
            s_ev, e_ev = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s_ev.record(stream)
            for _ in range(steps):
                g.replay()
            e_ev.record(stream)
        torch.cuda.synchronize()
        dist.barrier()
        if plans:
            ms = s_ev.elapsed_time(e_ev) / steps
            # end to end: pinned host f in, replay, y out, every step
            fh = [f.cpu().pin_memory() for f in f32s]
            yh = [torch.empty(f.shape, dtype=f.dtype).pin_memory() for f in f32s]
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            for _ in range(steps):
                for h, d_ in zip(fh, f32s):
                    d_.copy_(h, non_blocking=True)
                g.replay()
                for h, d_ in zip(yh, y32s):
                    h.copy_(d_, non_blocking=True)
                torch.cuda.synchronize()
            e2e_ms = (time.perf_counter() - t0) / steps * 1e3
        local_dof = sum(p.dof for p in plans)
        red = torch.tensor([ms, e2e_ms], dtype=torch.float64, device=dev)
        dist.all_reduce(red, op=dist.ReduceOp.MAX)
        tot = torch.tensor([float(local_dof), flops, float(len(plans))], dtype=torch.float64, device=dev)
        dist.all_reduce(tot, op=dist.ReduceOp.SUM)
        ms, e2e_ms = float(red[0]), float(red[1])
        dof, flops_all, nprob = float(tot[0]), float(tot[1]), int(tot[2])
        if rank == 0:
            line = {
                "metric": METRIC, "value": dof / (ms * 1e-3) / 1e9, "unit": UNIT, "n_gpus": world,
                "steps": steps, "warmup": max(3, args.warmup), "ms_per_step": ms, "higher_is_better": True,
                "scaling": "strong", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (dense N(0,1/deg) operators, f ~ N(0,1), seed 3)",
                "config": {"workload": "batched: %d problems, d in {2,3,4}, SG lev 3..%d, deg 2..4, all pairs"
                                       % (args.batch_problems, args.batch_max_level),
                           "dof": int(dof), "problems": nprob, "flops_per_step": flops_all,
                           "parallelism": "problem shards over %d ranks by cost, no data-path collective" % world,
                           "launch": "one persistent launch per rank, replayed from a CUDA graph",
                           "tuned_rank0": info},
                "compute": {"gflops_per_s": flops_all / (ms * 1e-3) / 1e9},
                "e2e": {"value": dof / (e2e_ms * 1e-3) / 1e9, "unit": UNIT, "h2d_bytes_per_step": int(4 * dof),
                        "d2h_bytes_per_step": int(4 * dof), "ms_per_step": e2e_ms},
                "gpu_launches": steps * 2 * world,
            }
            print(json.dumps(line), flush=True)
        for p in plans:
            p.close()
    finally:
        dist.destroy_process_group()


def run_implicit(args, rank, local):
    """The implicit configuration alone (rank 0): diffusion2 SG 8, deg 4, ten backward-Euler
    steps, mixed and FP64 (see implicit_steps); one JSON line, time per step (lower is
    better)."""
    import torch

    if rank != 0:
        return
    torch.cuda.set_device(local)
    out = implicit_steps(torch.device("cuda", local))
    line = {
        "metric": "backward-Euler step time, mixed-precision GMRES(30)-IR to 1e-10", "impl": "ours",
        "value": out["mixed"]["ms_per_step"], "unit": "ms/step", "n_gpus": 1, "steps": 10, "warmup": 1,
        "ms_per_step": out["mixed"]["ms_per_step"], "higher_is_better": False, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 inner / f64 outer",
        "data": "synthetic (projection of sin(pi x) sin(pi y) + 1e-3 N(0,1), seed 2)",
        "config": {"workload": "diffusion2 LDG, SG lev 8, deg 4, dt = h^2, Dirichlet zero", "dof": out["dof"]},
        "variants": out,
    }
    print(json.dumps(line), flush=True)


def gather_stream(plan, f32, flush, stream, steps=50):
    """The L2-to-SM rate of the plan's own gather pattern: every work entry's column block
    streamed into shared memory with the apply's bulk copies and no arithmetic
    (asg_probe_gather_f32), L2 flushed before each launch as for the apply.  Best stage count."""
    import ctypes as C

    import torch
    from asgkron._lib import check, lib

    out = torch.empty(plan.N, dtype=torch.float32, device=f32.device)
    st = plan.stats()
    gbytes = st["num_entries"] * plan.B * 4
    res = {}
    for stages in (2, 4, 8):
        def launch():
            check(lib().asg_probe_gather_f32(plan.handle, C.c_void_p(f32.data_ptr()), C.c_void_p(out.data_ptr()),
                                             stages, C.c_void_p(stream.cuda_stream)))
        for _ in range(3):
            flush()
            launch()
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        for s, e in ev:
            flush()
            s.record(stream)
            launch()
            e.record(stream)
        torch.cuda.synchronize()
        ms = sum(s.elapsed_time(e) for s, e in ev) / steps
        res["stages_%d" % stages] = {"ms": ms, "gbs": gbytes / (ms * 1e-3) / 1e9}
    best = min(res.values(), key=lambda r: r["ms"])
    return {"gather_bytes_per_launch": gbytes, "ms": best["ms"], "gbs": best["gbs"], "by_stages": res}


def fma_peaks(dev, stream):
    """FP32 paired-FMA and FP64 FMA issue peaks of this GPU (asg_probe_fma: 152 x 8 CTAs of 256
    threads, 8 independent chains each), TFLOP/s."""
    import ctypes as C

    import torch
    from asgkron._lib import check, lib

    out = torch.zeros(2, dtype=torch.float64, device=dev)
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    res = {}
    for prec, name, iters in ((1, "fp32_ffma2_tflops", 40000), (0, "fp64_dfma_tflops", 4000)):
        flops = C.c_double(0)
        def launch():
            check(lib().asg_probe_fma(prec, nsm * 8, iters, C.c_void_p(out.data_ptr()), C.byref(flops),
                                      C.c_void_p(stream.cuda_stream)))
        launch()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(3):
            launch()
        e.record(stream)
        torch.cuda.synchronize()
        res[name] = 3 * flops.value / (s.elapsed_time(e) * 1e-3) / 1e12
    return res


def graph_replay(plan, f, y, stream, n_apply=100, reps=10):
    """n_apply back-to-back applies captured in one CUDA graph (no flush between them: the
    operands stay in L2), replayed reps times; returns microseconds per apply."""
    import torch

    for _ in range(3):
        plan.apply(f, y, stream)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        for _ in range(n_apply):
            plan.apply(f, y, stream)
    with torch.cuda.stream(stream):  # replay on the stream the events are recorded on
        g.replay()
        torch.cuda.synchronize()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        for _ in range(reps):
            g.replay()
        e.record(stream)
    torch.cuda.synchronize()
    return 1e3 * s.elapsed_time(e) / (reps * n_apply)


def small_config_graph(dev):
    """CPU-runnable configuration: continuity2 SG 4, deg 2 (48 elements, 192 DOF), FP64, f ~
    N(0,1) seed 0; 100 applies per CUDA graph (a single apply lasts microseconds)."""
    import numpy as np
    import torch

    import asgkron
    from asgkron import pdes

    pde = pdes.continuity2(4)
    idx = asgkron.hash_table_sparse_nD(pde.levels, 8).idx1d()
    plan = asgkron.Plan.create(pde.term_mats(2), idx, 2)
    f = torch.from_numpy(np.random.default_rng(0).standard_normal(plan.dof)).to(dev)
    y = torch.empty_like(f)
    stream = torch.cuda.Stream(dev)
    us = graph_replay(plan, f, y, stream)
    out = {"dof": plan.dof, "us_per_apply": us, "value": plan.dof / (us * 1e-6) / 1e9,
           "kernel": asgkron._lib.KERNEL_NAMES[plan.stats()["kernel_kind"]]}
    # the configuration's five explicit RK3 steps at CFL 0.01 (sources included), one step
    # captured in a CUDA graph and replayed five times per timed pass, each replay after the
    # upload of its stage times' source factors
    from asgkron.steppers import RK3Stepper

    dt = pde.dt(0.01)
    x = f.clone()
    stepper = RK3Stepper(plan, pde, idx)
    stepper.capture(x, dt)
    for i in range(5):
        stepper.replay(i * dt)
    torch.cuda.synchronize()
    ts = []
    for _ in range(20):
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record()
        for i in range(5):
            stepper.replay(i * dt)
        t1.record()
        torch.cuda.synchronize()
        ts.append(t0.elapsed_time(t1) * 1e3 / 5)
    out["rk3_step_us"] = statistics.median(ts)
    out["rk3_launches_per_step"] = 1  # sources, three applies and the stage updates in one cooperative launch
    plan.close()
    return out


def run_sharded(args, rank, world, local):
    """The headline workload on ``world`` GPUs with y = A f split by output element (strong
    scaling: the total work is the one-GPU workload).  Rows are split into contiguous ranges
    balanced by work entries; every rank builds the row-slice plan of its range, holds f for
    its rows, and per step exchanges exactly the halo blocks its rows read (one NCCL
    all-to-all into buffers allocated once) and applies its slice.  value = all DOF over the
    slowest rank's step time; e2e adds each rank's host copies of its f rows and y rows."""
    import numpy as np
    import torch
    import torch.distributed as dist

    import asgkron
    from asgkron.shard import ShardedApply, partition_rows, row_plan

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if not dist.is_initialized():
        if world == 1:  # --sharded on one GPU: a one-rank group
            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            os.environ.setdefault("MASTER_PORT", "29531")
            dist.init_process_group("nccl", device_id=dev, rank=0, world_size=1)
        else:
            dist.init_process_group("nccl", device_id=dev)
    pde, deg, idx, mats = build_workload()
    N, D = idx.shape
    B = deg ** D
    dof = N * B
    full = asgkron.Plan.create(mats, idx, deg)
    cost = full.row_entries()
    full.close()
    ranges = partition_rows(cost, world)
    r0, r1 = ranges[rank]
    plan = row_plan(mats, idx, deg, (r0, r1))
    sh = ShardedApply(plan, ranges, B)
    f_all = np.random.default_rng(4).standard_normal(dof).astype(np.float32)
    f_local = torch.from_numpy(f_all[r0 * B:r1 * B].copy()).to(dev)
    y = torch.empty(plan.dof, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream(dev)
    flush_buf = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)
    for _ in range(max(3, args.warmup)):
        flush_buf.fill_(1)
        sh.apply(f_local, y)
    sampler = ClockSampler(local)
    dist.barrier()
    torch.cuda.synchronize()
    t0 = time.time()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for s_, e_ in ev:
        flush_buf.fill_(1)
        s_.record(stream)
        sh.apply(f_local, y)
        e_.record(stream)
    torch.cuda.synchronize()
    dist.barrier()
    t1 = time.time()
    clocks = sampler.stop(t0, t1)
    ms = sum(s_.elapsed_time(e_) for s_, e_ in ev) / len(ev)
    t = torch.tensor([ms], device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    step_ms = float(t.item())
    # end to end: each rank's f rows in from pinned host memory, exchange, apply, y rows out
    fh = torch.from_numpy(f_all[r0 * B:r1 * B].copy()).pin_memory()
    yh = torch.empty(plan.dof, dtype=torch.float32).pin_memory()
    e2e_steps = max(1, min(args.steps, 200))
    for _ in range(3):
        f_local.copy_(fh, non_blocking=True)
        yh.copy_(sh.apply(f_local, y), non_blocking=True)
    torch.cuda.synchronize()
    dist.barrier()
    ta = time.perf_counter()
    for _ in range(e2e_steps):
        f_local.copy_(fh, non_blocking=True)
        yh.copy_(sh.apply(f_local, y), non_blocking=True)
    torch.cuda.synchronize()
    e2e_local = (time.perf_counter() - ta) / e2e_steps * 1e3
    t = torch.tensor([e2e_local], device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    e2e_ms = float(t.item())
    halo = torch.tensor([float(sh.halo.size)], device=dev)
    dist.all_reduce(halo)
    # roofline as on one GPU: the job's compulsory bytes (f read, y written, operators, pair
    # list) over the slowest rank's step, against the ranks' summed measured HBM bandwidth
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = float(json.load(open(peaks_path))["hbm_gbs"]) * world, "of measured (x %d GPUs)" % world
    else:
        peak, peak_src = FALLBACK_HBM_GBS * world, "of fallback (x %d GPUs)" % world
    alg = algorithmic_bytes(4, dof, len(mats), D, np.asarray(mats[0][0]).shape[0], N, N * N)
    achieved = alg / (step_ms * 1e-3) / 1e9
    if rank == 0:
        print(json.dumps({
            "metric": METRIC, "value": dof / (step_ms * 1e-3) / 1e9, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True,
            "scaling": "strong", "vs_baseline": None, "dtype": "f32", "data": DATA, "config": workload_config(dof),
            "details": {"parallelism": "row slices over %d ranks (balanced by work entries), halo all-to-all per "
                                       "step" % world,
                        "ranges": [[int(a), int(b)] for a, b in ranges],
                        "halo_blocks_total": int(halo.item()), "all_gather_blocks_would_be": (world - 1) * N},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": None, "peak_source": peak_src, "algorithmic_bytes_per_launch": alg},
            "e2e": {"value": dof / (e2e_ms * 1e-3) / 1e9, "unit": UNIT, "h2d_bytes_per_step": 4 * dof,
                    "d2h_bytes_per_step": 4 * dof, "ms_per_step": e2e_ms},
            "gpu_launches": args.steps * world,
            "clocks": clocks,
        }), flush=True)
    plan.close()
    dist.destroy_process_group()


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
        return
    if args.workload == "batched":
        if world > 1:
            run_batched_sharded(args, rank, world, local)
        else:
            run_batched(args, rank, local)
        return
    if args.workload == "implicit":
        run_implicit(args, rank, local)
        return
    if (world > 1 and not args.replicas) or args.sharded:
        run_sharded(args, rank, world, local)
        return
    import numpy as np
    import torch

    import asgkron

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    pg = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
        pg = dist
    pde, deg, idx, mats = build_workload()
    N, D = idx.shape
    T = pde.num_terms
    B = deg ** D
    dof = N * B
    n1d = deg * 2 ** 4
    stream = torch.cuda.current_stream(dev)

    plan = asgkron.Plan.create(mats, idx, deg, structure="detect")
    st = plan.stats()
    rng = np.random.default_rng(4 + rank)
    f64_h = rng.standard_normal(dof)
    f32 = torch.from_numpy(f64_h.astype(np.float32)).to(dev)
    y32 = torch.empty_like(f32)
    flush_buf = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device=dev)
    ctr = [0]

    def flush():
        ctr[0] = (ctr[0] + 1) & 0xFF
        flush_buf.fill_(ctr[0])

    # ---- timed region: K FP32 applies, L2 flushed before each ---------------------------
    sampler = ClockSampler(local)
    for _ in range(args.warmup):
        flush()
        plan.apply(f32, y32, stream)
    if pg:
        pg.barrier()
    torch.cuda.synchronize()
    t0 = time.time()
    ms = time_device(plan, f32, y32, flush, args.steps, 0, stream)
    torch.cuda.synchronize()
    if pg:
        pg.barrier()
    t1 = time.time()
    clocks = sampler.stop(t0, t1)
    apply_ms = sum(ms) / len(ms)
    if pg:
        t = torch.tensor([apply_ms], device=dev)
        pg.all_reduce(t, op=pg.ReduceOp.MAX)
        apply_ms = float(t.item())
    value = world * dof / (apply_ms * 1e-3) / 1e9

    # ---- end to end through the host-pointer C ABI call ----------------------------------
    # asg_apply_host_f32 on page-locked host f and y (the call a host caller makes; ctypes
    # arguments prepared once), L2 flushed and the device idle before each call
    import ctypes as C

    from asgkron._lib import check, lib

    fh = torch.from_numpy(f64_h.astype(np.float32)).pin_memory()
    yh = torch.empty_like(fh).pin_memory()
    host_fn, h_args = lib().asg_apply_host_f32, (plan.handle, C.c_void_p(fh.data_ptr()), C.c_void_p(yh.data_ptr()))
    for _ in range(max(3, args.warmup)):
        check(host_fn(*h_args))
    e2e_steps = max(1, min(args.steps, 500))
    e2e_t = []
    for _ in range(e2e_steps):
        flush()
        torch.cuda.synchronize()
        t_a = time.perf_counter()
        check(host_fn(*h_args))
        e2e_t.append(time.perf_counter() - t_a)
    # host-timed: the median, so that a stall of the host process does not stand for the call
    e2e_ms = statistics.median(e2e_t) * 1e3
    e2e_mean_ms = sum(e2e_t) / len(e2e_t) * 1e3
    e2e_value = dof / (e2e_ms * 1e-3) / 1e9
    plan.apply(f32, y32, stream)
    torch.cuda.synchronize()
    e2e_matches_device = bool(torch.equal(yh, y32.cpu()))

    # ---- variants: FP64 (same work model) and the reference work model ------------------
    variants = {}
    y64 = None
    if not args.skip_variants:
        f64 = torch.from_numpy(f64_h).to(dev)
        y64 = torch.empty_like(f64)
        ms64 = time_device(plan, f64, y64, flush, max(5, min(args.steps, 200)), 3, stream)
        fp64_ms = sum(ms64) / len(ms64)
        plan.apply(f32, y32, stream)
        torch.cuda.synchronize()
        err = float(torch.linalg.norm(y32.double() - y64) / torch.linalg.norm(y64))
        variants["fp64_structured"] = {"value": dof / (fp64_ms * 1e-3) / 1e9, "ms": fp64_ms,
                                       "fp32_speedup": fp64_ms / apply_ms}
        variants["fp32_rel_err_vs_fp64"] = err
        dense = asgkron.Plan.create(mats, idx, deg, structure="none")
        msd = time_device(dense, f32, y32, flush, 3, 1, stream)
        dms = sum(msd) / len(msd)
        dst = dense.stats()
        variants["fp32_reference_work_model"] = {
            "value": dof / (dms * 1e-3) / 1e9, "ms": dms, "entries": dst["num_entries"],
            "gflops_per_s": dst["flops_reference"] / (dms * 1e-3) / 1e9}
        dense.close()
        ystar = torch.from_numpy(np.random.default_rng(5).standard_normal(dof).astype(np.float32)).to(dev)
        variants["fp32_forward_backward"] = forward_backward(plan, f32, ystar, flush, max(5, min(args.steps, 200)),
                                                             stream, dof, n1d)
        gstream = torch.cuda.Stream(dev)
        variants["fp32_graph_100_applies_l2_resident"] = {
            "us_per_apply": graph_replay(plan, f32, y32, gstream)}
        variants["fp32_graph_100_applies_l2_resident"]["value"] = (
            dof / (variants["fp32_graph_100_applies_l2_resident"]["us_per_apply"] * 1e-6) / 1e9)
        variants["continuity2_lev4_deg2_fp64_graph"] = small_config_graph(dev)
        variants["implicit_diffusion2_lev8_deg4"] = implicit_steps(dev)
        variants["precision_continuity3_lev6_deg3"] = precision_continuity3(dev, flush, stream)
        variants["adaptive_plan_updates_continuity2"] = adaptive_plan_updates(dev)
        variants["batched_256_lev3_7"] = batched_measure(dev, 256, 7, max(1, min(args.steps, 5)), 3)
        # the roofline denominators measured here: the plan's gather pattern and the FMA pipes
        gs = gather_stream(plan, f32, flush, stream)
        gs["apply_frac_of_gather_stream"] = gs["ms"] / apply_ms
        variants["gather_stream"] = gs
        peaks = fma_peaks(dev, stream)
        rw = variants["fp32_reference_work_model"]
        peaks["fp32_reference_work_model_frac"] = rw["gflops_per_s"] / 1e3 / peaks["fp32_ffma2_tflops"]
        f64_flops = st["flops_executed"] / (fp64_ms * 1e-3) / 1e12
        peaks["fp64_structured_tflops"] = f64_flops
        peaks["fp64_structured_frac"] = f64_flops / peaks["fp64_dfma_tflops"]
        variants["fma_peaks"] = peaks
        # the autotuner on the headline plan (per precision; then back to the default)
        variants["tuner"] = {"fp32": plan.tune("float32"), "fp64": plan.tune("float64")}
        plan.set_kernel(st["kernel_kind"])
        # end to end through the FP64 host-pointer call (what the MATLAB gateway makes)
        f64h = torch.from_numpy(np.ascontiguousarray(f64_h)).pin_memory()
        y64h = torch.empty_like(f64h).pin_memory()
        h64 = (plan.handle, C.c_void_p(f64h.data_ptr()), C.c_void_p(y64h.data_ptr()))
        for _ in range(3):
            check(lib().asg_apply_host_f64(*h64))
        t64 = []
        for _ in range(max(5, min(args.steps, 100))):
            flush()
            torch.cuda.synchronize()
            t_a = time.perf_counter()
            check(lib().asg_apply_host_f64(*h64))
            t64.append(time.perf_counter() - t_a)
        e64 = statistics.median(t64) * 1e3
        variants["e2e_fp64_host"] = {"ms_per_step": e64, "mean_ms": sum(t64) / len(t64) * 1e3,
                                     "max_ms": max(t64) * 1e3, "slowest_call": int(max(range(len(t64)), key=t64.__getitem__)),
                                     "value": dof / (e64 * 1e-3) / 1e9, "statistic": "median of host-timed calls",
                                     "h2d_bytes_per_step": 8 * dof, "d2h_bytes_per_step": 8 * dof}

    # ---- roofline ------------------------------------------------------------------------
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "of measured"
    else:
        peak, peak_src = FALLBACK_HBM_GBS, "of fallback"
    alg = algorithmic_bytes(4, dof, T, D, n1d, N, st["num_pairs"])
    achieved = alg / (apply_ms * 1e-3) / 1e9
    if "fp32_forward_backward" in variants:
        fb = variants["fp32_forward_backward"]
        fb["frac_hbm"] = fb["achieved_gbs"] / peak
    traffic = gather_ncu = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        tj = json.load(open(tpath))
        traffic = tj.get("k_single_tma_fp32_continuity6")
        gather_ncu = tj.get("k_single_tma_fp32_continuity6_l2_to_sm")
    # second roofline: the L2-to-SM bytes the kernel moves (ncu) over the rate the same kind of
    # gather reaches when streamed alone (asg_probe_gather_f32, measured in this run)
    gather_roof = None
    if gather_ncu and "gather_stream" in variants:
        g_ach = gather_ncu / (apply_ms * 1e-3) / 1e9
        g_peak = variants["gather_stream"]["gbs"]
        gather_roof = {"achieved": g_ach, "peak": g_peak, "unit": "GB/s", "frac": g_ach / g_peak,
                       "bytes_per_launch": gather_ncu,
                       "peak_source": "measured in this run: the plan's gather pattern streamed alone"}

    cpu = None
    if rank == 0 and world == 1:
        cpu = cpu_baseline(f64_h)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": apply_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": DATA,
            "config": workload_config(dof),
            "details": {"work_model": "structured (zero blocks skipped, identity factors as copies; drop_tol %.0e)"
                                      % asgkron.DEFAULT_DROP_TOL,
                        "entries": st["num_entries"], "kernel": asgkron._lib.KERNEL_NAMES[st["kernel_kind"]],
                        "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                         "algorithmic_bytes_per_launch": alg, "gather": gather_roof},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": dof * 4, "d2h_bytes_per_step": dof * 4,
                    "ms_per_step": e2e_ms, "mean_ms": e2e_mean_ms, "max_ms": max(e2e_t) * 1e3,
                    "statistic": "median of host-timed calls",
                    "call": "asg_apply_host_f32, page-locked f and y",
                    "equals_device_apply": e2e_matches_device},
            "gpu_launches": args.steps,
            "clocks": clocks,
            "variants": variants,
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    plan.close()
    if pg:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
