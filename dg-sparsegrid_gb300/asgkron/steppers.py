"""Time steppers on the GPU operator application (time_advance.m).

* ``RK3Stepper``  RungeKutta3 (time_advance.m:151-204): separable sources s(t) = sum_s c_s(t)
  v_s are formed on the device from precomputed spatial parts; one step (three source
  combinations + three applies + three fused stage updates) can be captured once into a CUDA
  graph and replayed, with only the time factors copied in before each replay.
* ``be_solve`` / ``be_step``  backward Euler (time_advance.m:267-349): (I - dt A) f1 =
  f0 + dt s solved matrix-free by GMRES inside iterative refinement (asg_be_solve).

torch provides device memory, streams and the graph object; every kernel is libasgkron's.
"""
import ctypes as C

import numpy as np

from ._lib import GmresInfo, GmresOpts, check, lib


class RK3Stepper:
    def __init__(self, plan, pde=None, idx1d=None, dtype="float64", source_parts=None, time_factors=None):
        import torch

        self.plan = plan
        self.torch_dtype = torch.float64 if dtype in ("float64", torch.float64) else torch.float32
        self.n = plan.dof
        dev = torch.device("cuda")
        if source_parts is None and pde is not None:
            # sources and boundary data: both enter each stage as rhs (time_advance.m:158-190)
            source_parts, time_factors = pde.forcing_parts(plan.deg, np.asarray(idx1d))
        self.tfac = list(time_factors or [])
        ns = len(self.tfac)
        self.ns = ns
        self.vecs = [torch.from_numpy(np.asarray(v, dtype=np.float64)).to(dev) for v in (source_parts or [])]
        self.vec_ptrs = torch.tensor([v.data_ptr() for v in self.vecs] or [0], dtype=torch.int64, device=dev)
        self.coef = torch.zeros(3 * max(ns, 1), dtype=torch.float64, device=dev)
        # a ring of page-locked sources for the time factors: a replay queued while an earlier
        # one's copy has not run yet must not overwrite that copy's source
        self.coef_ring = [torch.zeros(3 * max(ns, 1), dtype=torch.float64).pin_memory() for _ in range(4)]
        self.coef_np = [r.numpy() for r in self.coef_ring]  # written in place, no tensor per step
        self.coef_done = [torch.cuda.Event() for _ in range(4)]
        self.coef_used = [False] * 4
        self._slot = 0
        per = 16 // (8 if self.torch_dtype == torch.float64 else 4)  # values per 16 bytes
        self.work = torch.empty(4 * ((self.n + per - 1) // per * per), dtype=self.torch_dtype, device=dev)
        self.graph = None
        self._f_static = None

    def _set_time(self, t, dt):
        if self.ns == 0:
            return
        k = self._slot
        if self.coef_used[k]:
            self.coef_done[k].synchronize()
        self.coef_np[k][:] = [fn(tt) for tt in (t, t + 0.5 * dt, t + dt) for fn in self.tfac]
        self.coef.copy_(self.coef_ring[k], non_blocking=True)
        self.coef_done[k].record()
        self.coef_used[k] = True
        self._slot = (k + 1) % len(self.coef_ring)

    def _launch(self, f, dt, stream):
        # the stage sources (sum of the spatial parts times their time factors, read from the
        # device) are formed inside the step
        fn = lib().asg_rk3_step_sources_f64 if self.torch_dtype.itemsize == 8 else lib().asg_rk3_step_sources_f32
        check(fn(self.plan.handle, C.c_void_p(f.data_ptr()), float(dt), self.ns, C.c_void_p(self.coef.data_ptr()),
                 C.c_void_p(self.vec_ptrs.data_ptr()), C.c_void_p(self.work.data_ptr()),
                 self.work.numel() * self.work.element_size(), C.c_void_p(stream.cuda_stream)))

    def step(self, f, t, dt):
        """Advance f (CUDA tensor, in place) from t to t + dt."""
        import torch

        self._set_time(t, dt)
        self._launch(f, dt, torch.cuda.current_stream())
        return f

    def capture(self, f, dt):
        """Capture one step on the static tensor f into a CUDA graph (dt fixed)."""
        import torch

        self._f_static = f
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):  # warm-up outside the capture (kernel attributes, lazy state)
            saved = f.clone()
            self._launch(f, dt, s)
            f.copy_(saved)
        torch.cuda.current_stream().wait_stream(s)
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self._launch(f, dt, torch.cuda.current_stream())
        self._dt = dt
        return self.graph

    def replay(self, t):
        """One captured step from time t (the graph reads the time factors from the device)."""
        self._set_time(t, self._dt)
        self.graph.replay()
        return self._f_static


# GMRES precision modes (asg_gmres_opts.mixed): the outer residual, its norm and x are FP64 in
# all three; "matvec32" runs only the operator application in FP32 (the basis, the Arnoldi
# dot products and norms, the Givens rotations and the solution update stay FP64);
# "inner32" runs the whole inner cycle in FP32; "fp64" nothing.
GMRES_MODES = {"fp64": 0, "inner32": 1, "matvec32": 2}


def gmres_mode(mixed):
    """asg_gmres_opts.mixed for ``mixed``: a mode name, True (= "matvec32") or False (= "fp64")."""
    if mixed is True:
        return GMRES_MODES["matvec32"]
    if mixed is False or mixed is None:
        return GMRES_MODES["fp64"]
    if mixed not in GMRES_MODES:
        raise ValueError("mixed must be True, False or one of %s" % sorted(GMRES_MODES))
    return GMRES_MODES[mixed]


def be_solve(plan, dt, b, x, restart=30, tol=1e-10, max_outer=60, inner_reduction=1e-5, mixed=True):
    """Solve (I - dt A) x = b in place (FP64 CUDA tensors); returns the info dict.  ``mixed``
    selects the precision of the GMRES cycles (see GMRES_MODES; True = "matvec32")."""
    import torch

    opts = GmresOpts(int(restart), int(max_outer), float(tol), float(inner_reduction), gmres_mode(mixed))
    nbytes = C.c_size_t(0)
    check(lib().asg_be_workspace(plan.handle, C.byref(opts), C.byref(nbytes)))
    work = torch.empty(max(1, nbytes.value), dtype=torch.uint8, device=x.device)
    info = GmresInfo()
    check(lib().asg_be_solve(plan.handle, float(dt), C.c_void_p(b.data_ptr()), C.c_void_p(x.data_ptr()), C.byref(opts),
                             C.byref(info), C.c_void_p(work.data_ptr()), nbytes.value,
                             C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return {k: getattr(info, k) for k, _ in GmresInfo._fields_}


def be_step(plan, f0, dt, source=None, **kw):
    """f1 for backward Euler: (I - dt A) f1 = f0 + dt * source, initial guess f0."""
    b = f0.clone() if source is None else f0 + dt * source
    x = f0.clone()
    info = be_solve(plan, dt, b, x, **kw)
    return x, info
