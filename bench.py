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
(asg_apply_host_f32: H2D of f from pinned memory, apply, D2H of y, synchronise);
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
FALLBACK_HBM_GBS = 6800.0


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-rows", type=int, default=48, help="rows in the bounded CPU sample")
    ap.add_argument("--skip-variants", action="store_true")
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


def cpu_baseline(mats, idx, deg, f64, rows):
    from oracle import cref

    import numpy as np

    cores = os.cpu_count() or 1
    sel = np.linspace(0, idx.shape[0] - 1, rows).astype(np.int32)
    cref.apply_rows(mats, idx, deg, f64, rows=sel[:2], nthreads=cores)  # warm (build, page-in)
    t0 = time.perf_counter()
    cref.apply_rows(mats, idx, deg, f64, rows=sel, nthreads=cores)
    dt = time.perf_counter() - t0
    B = deg ** idx.shape[1]
    return {"value": rows * B / dt / 1e9, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": "%d of %d rows, reference loop (all pairs x 6 terms x 6-mode chain), FP64, %.2f s" %
                      (rows, idx.shape[0], dt)}


def run_reference(args, rank):
    """Time the CPU implementation of the path (C restatement of the reference loop) on the
    host cores.  One step is a bounded sample of the workload: ``rows`` row elements x a
    contiguous chunk of ``ncols`` column elements each, sized from a calibration step so that
    warmup + steps stay within ~90 s; the rate is scaled to DOF of complete rows (a row needs
    all N columns)."""
    import numpy as np

    if rank != 0:
        return
    from oracle import cref

    pde, deg, idx, mats = build_workload()
    N = idx.shape[0]
    B = deg ** idx.shape[1]
    f64 = np.random.default_rng(4).standard_normal(N * B)
    cores = os.cpu_count() or 1
    rows = np.linspace(0, N - 1, min(N, max(cores, 1))).astype(np.int32)

    def csr(ncols, shift):
        rp = np.zeros(N + 1, dtype=np.int64)
        cols = []
        for r in rows:
            c0 = (int(r) * 7 + shift) % N
            cc = [(c0 + k) % N for k in range(ncols)]
            cols.extend(cc)
            rp[r + 1] = ncols
        return np.cumsum(rp), np.array(cols, dtype=np.int32)

    # calibrate: seconds per (row, column) pair with all threads busy
    t0 = time.perf_counter()
    cref.apply_rows(mats, idx, deg, f64, rows=rows, pairs0=csr(8, 0), nthreads=cores)
    per_pair = (time.perf_counter() - t0) / (rows.size * 8)
    steps = max(1, args.steps)
    total = steps + max(args.warmup, 0)
    t_step = min(2.0, max(0.005, 90.0 / total))
    ncols = int(max(1, min(N, t_step / (per_pair * rows.size))))
    pairs = [csr(ncols, k) for k in range(4)]
    for k in range(max(args.warmup, 0)):
        cref.apply_rows(mats, idx, deg, f64, rows=rows, pairs0=pairs[k % 4], nthreads=cores)
    t_all = 0.0
    for k in range(steps):
        t0 = time.perf_counter()
        cref.apply_rows(mats, idx, deg, f64, rows=rows, pairs0=pairs[k % 4], nthreads=cores)
        t_all += time.perf_counter() - t0
    per_step = t_all / steps
    row_equiv = rows.size * ncols / N
    value = row_equiv * B / per_step / 1e9
    sample = "%d rows x %d of %d columns per step (all 6 terms, 6-mode chain), FP64" % (rows.size, ncols, N)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus, "steps": steps,
        "warmup": args.warmup, "ms_per_step": per_step * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (f ~ N(0,1), seed 4)",
        "config": {"workload": WORKLOAD, "step": "bounded sample: " + sample,
                   "implementation": "C restatement of apply_A.m's loop, OpenMP over rows "
                                     "(the MATLAB reference cannot run on the box)",
                   "l2": "host-only"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
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


def main():
    args = parse_args()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank)
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
    fh = torch.from_numpy(f64_h.astype(np.float32)).pin_memory()
    yh = torch.empty_like(fh).pin_memory()
    fh_np, yh_np = fh.numpy(), yh.numpy()
    for _ in range(max(3, args.warmup)):
        plan.apply_host(fh_np, yh_np)
    e2e_steps = max(1, min(args.steps, 500))
    tot = 0.0
    for _ in range(e2e_steps):
        flush()
        torch.cuda.synchronize()
        t_a = time.perf_counter()
        plan.apply_host(fh_np, yh_np)
        tot += time.perf_counter() - t_a
    e2e_ms = tot / e2e_steps * 1e3
    e2e_value = dof / (e2e_ms * 1e-3) / 1e9

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

    # ---- roofline ------------------------------------------------------------------------
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak = float(json.load(open(peaks_path))["hbm_gbs"])
        peak_src = "of measured"
    else:
        peak, peak_src = FALLBACK_HBM_GBS, "of fallback"
    alg = algorithmic_bytes(4, dof, T, D, n1d, N, st["num_pairs"])
    achieved = alg / (apply_ms * 1e-3) / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        traffic = json.load(open(tpath)).get("k_single_mode_fp32_continuity6")

    cpu = None
    if rank == 0 and world == 1:
        cpu = cpu_baseline(mats, idx, deg, f64_h, max(1, args.cpu_rows))

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": apply_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (continuity6 operators from the DG builder; f ~ N(0,1) seed 4)",
            "config": {"workload": WORKLOAD, "dof": dof, "work_model": "structured (zero blocks skipped, identity "
                       "factors as copies; drop_tol %.0e)" % asgkron.DEFAULT_DROP_TOL,
                       "entries": st["num_entries"], "kernel": asgkron._lib.KERNEL_NAMES[st["kernel_kind"]],
                       "l2": "flushed before every step (512 MB write, outside the timed apply)",
                       "parallelism": "replicas" if world > 1 else "single GPU"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                         "algorithmic_bytes_per_launch": alg},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": dof * 4, "d2h_bytes_per_step": dof * 4,
                    "ms_per_step": e2e_ms},
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
