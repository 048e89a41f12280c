"""Host-side mirror of the reference's operator-application interface.

``Plan`` wraps one ``asg_plan`` (operators + element 1-D indices + pair list) and applies
``y = A*f`` on the GPU, either on device tensors (torch CUDA tensors are used only as
device memory and stream handles) or on host arrays.  ``apply_A`` keeps the MATLAB
signature of apply_A.m:1 and caches plans the way a MEX gateway would keep a persistent
handle.
"""
import ctypes as C

import numpy as np

from ._lib import (ASG_STRUCT_DETECT, ASG_STRUCT_NONE, PlanDesc, PlanExt, PlanStats, check, lib)

# |entry| <= DEFAULT_DROP_TOL * max|op| is treated as an exact zero by the structure
# analysis.  The wavelet-space mass factors differ from the identity by ~1e-15 relative
# (rotation round-off), which this threshold absorbs; the induced change of y is far
# below the 1e-12 FP64 parity bound.
DEFAULT_DROP_TOL = 1e-13


def _as_term_mats(term_mats):
    out = []
    for row in term_mats:
        out.append([np.asfortranarray(np.asarray(m, dtype=np.float64)) for m in row])
    return out


class Plan:
    """y = A f for fixed operators, element indices and pair list.

    term_mats: T lists of d dense 1-D operators (pde.terms{t}.terms_1D{d}.mat).
    idx1d:     [N, d] 1-D indices (A_data.element_local_index_D), base ``index_base``.
    pairs:     None (all pairs, the apply_A default) or (row_ptr, cols) CSR.
    structure: "none" (reference work model) or "detect" (skip zero blocks, identity
               factors as copies; ``drop_tol`` relative threshold).
    """

    def __init__(self, term_mats, idx1d, pairs=None, structure="detect", drop_tol=DEFAULT_DROP_TOL, index_base=1):
        mats = _as_term_mats(term_mats)
        idx = np.ascontiguousarray(np.asarray(idx1d, dtype=np.int32))
        if idx.ndim != 2:
            raise ValueError("idx1d must be [num_elems, num_dims]")
        N, D = idx.shape
        T = len(mats)
        if T == 0 or any(len(r) != D for r in mats):
            raise ValueError("term_mats must hold num_terms lists of num_dims operators")
        deg = None
        self.term_mats = mats
        self.structure = structure
        self.N, self.D, self.T = N, D, T
        self._keep = [mats, idx]
        ptrs = (C.POINTER(C.c_double) * (T * D))()
        lds = (C.c_int * (T * D))()
        for t in range(T):
            for d in range(D):
                m = mats[t][d]
                if m.ndim != 2 or m.shape[0] != m.shape[1]:
                    raise ValueError("operator (term %d, dim %d) must be square" % (t, d))
                ptrs[t * D + d] = m.ctypes.data_as(C.POINTER(C.c_double))
                lds[t * D + d] = m.shape[0]
        self._ptrs, self._lds = ptrs, lds
        desc = PlanDesc()
        desc.num_dims = D
        desc.num_terms = T
        desc.num_elems = N
        desc.index_base = int(index_base)
        desc.idx1d = idx.ctypes.data_as(C.POINTER(C.c_int))
        if pairs is not None:
            rp = np.ascontiguousarray(np.asarray(pairs[0], dtype=np.int64))
            cl = np.ascontiguousarray(np.asarray(pairs[1], dtype=np.int32))
            if cl.size == 0:
                cl = np.zeros(1, dtype=np.int32)
            self._keep += [rp, cl]
            desc.row_ptr = rp.ctypes.data_as(C.POINTER(C.c_longlong))
            desc.cols = cl.ctypes.data_as(C.POINTER(C.c_int))
        desc.ops = ptrs
        desc.op_ld = lds
        desc.structure = ASG_STRUCT_DETECT if structure == "detect" else ASG_STRUCT_NONE
        desc.drop_tol = float(drop_tol) if structure == "detect" else 0.0
        self.deg = deg
        self._desc = desc
        self._handle = C.c_void_p()

    def _create(self, deg, rows=None, op_blocks=None):
        self._desc.deg = int(deg)
        self.deg = int(deg)
        self.B = self.deg ** self.D
        self.rows = None
        if rows is None and op_blocks is None:
            check(lib().asg_plan_create(C.byref(self._desc), C.byref(self._handle)))
        else:
            ext = PlanExt()
            r0, r1 = (0, self.N) if rows is None else (int(rows[0]), int(rows[1]))
            ext.row_begin, ext.row_end = r0, r1
            if op_blocks is not None:
                ob = np.ascontiguousarray(np.asarray(op_blocks, dtype=np.int32))
                if ob.shape != (self.D,):
                    raise ValueError("op_blocks must hold num_dims values")
                self._keep.append(ob)
                ext.op_blocks = ob.ctypes.data_as(C.POINTER(C.c_int))
            check(lib().asg_plan_create_ex(C.byref(self._desc), C.byref(ext), C.byref(self._handle)))
            if (r0, r1) != (0, self.N):
                self.rows = (r0, r1)
        n_out = self.N if self.rows is None else self.rows[1] - self.rows[0]
        self.dof = n_out * self.B                      # values of y
        self.dof_in = (n_out + len(self.halo())) * self.B  # values of f

    @classmethod
    def create(cls, term_mats, idx1d, deg, rows=None, op_blocks=None, **kw):
        """rows=(r0, r1): a row-slice plan (asg_plan_create_ex): y holds rows r0..r1-1, f holds
        those rows followed by ``halo()``.  op_blocks: per dimension, the 1-D blocks to pack
        (reserves room for ``update_elements`` with finer tables)."""
        p = cls(term_mats, idx1d, **kw)
        p._create(deg, rows=rows, op_blocks=op_blocks)
        return p

    def halo(self):
        """Table ids (in the plan's index base) of the input elements after a row slice's rows,
        in the order f holds them (empty for a whole-table plan)."""
        n = C.c_longlong(0)
        check(lib().asg_plan_halo(self._handle, None, 0, C.byref(n)))
        out = np.zeros(max(1, n.value), dtype=np.int32)
        if n.value:
            check(lib().asg_plan_halo(self._handle, out.ctypes.data_as(C.POINTER(C.c_int)), n.value, C.byref(n)))
        return out[:n.value]

    def row_entries(self):
        """Work entries of each output row (asg_plan_row_entries): the cost partition_rows
        balances."""
        out = np.zeros(max(1, self.dof // self.B), dtype=np.int64)
        check(lib().asg_plan_row_entries(self._handle, out.ctypes.data_as(C.POINTER(C.c_longlong))))
        return out[:self.dof // self.B]

    def update_elements(self, idx1d, pairs=None):
        """asg_plan_update_elements: a new element table (and pair list) on the plan's operators.
        Raises AsgError(ASG_ERR_CAPACITY) when a 1-D index lies beyond the packed operators."""
        idx = np.ascontiguousarray(np.asarray(idx1d, dtype=np.int32))
        if idx.ndim != 2 or idx.shape[1] != self.D:
            raise ValueError("idx1d must be [num_elems, num_dims]")
        rp_p = cl_p = None
        keep = [idx]
        if pairs is not None:
            rp = np.ascontiguousarray(np.asarray(pairs[0], dtype=np.int64))
            cl = np.ascontiguousarray(np.asarray(pairs[1], dtype=np.int32))
            if cl.size == 0:
                cl = np.zeros(1, dtype=np.int32)
            keep += [rp, cl]
            rp_p = rp.ctypes.data_as(C.POINTER(C.c_longlong))
            cl_p = cl.ctypes.data_as(C.POINTER(C.c_int))
        check(lib().asg_plan_update_elements(self._handle, idx.shape[0], idx.ctypes.data_as(C.POINTER(C.c_int)),
                                             rp_p, cl_p))
        self.N = idx.shape[0]
        self.dof = self.dof_in = self.N * self.B
        self._keep[1] = idx
        self._keep += keep

    # ---------------------------------------------------------------------------------
    @property
    def handle(self):
        return self._handle.value

    def stats(self):
        s = PlanStats()
        check(lib().asg_plan_stats_get(self._handle, C.byref(s)))
        return {k: getattr(s, k) for k, _ in PlanStats._fields_}

    def tune(self, dtype="float32", stream=None):
        """asg_plan_tune: time every kernel family for this plan in one precision and keep the
        fastest; returns {"kind", "name", "ms", "default_ms"}."""
        import torch

        prec = 1 if dtype in ("float32", torch.float32) else 0
        k, ms, dms = C.c_int(0), C.c_float(0), C.c_float(0)
        s = stream if stream is not None else torch.cuda.current_stream()
        check(lib().asg_plan_tune(self._handle, prec, C.c_void_p(s.cuda_stream), C.byref(k), C.byref(ms), C.byref(dms)))
        from ._lib import KERNEL_NAMES

        return {"kind": k.value, "name": KERNEL_NAMES[k.value], "ms": ms.value, "default_ms": dms.value}

    def kernel_for(self, dtype="float32"):
        """The kernel kind applies in this precision run (tuned or the plan's default)."""
        import torch

        k = C.c_int(0)
        check(lib().asg_plan_kernel_for(self._handle, 1 if dtype in ("float32", torch.float32) else 0, C.byref(k)))
        return k.value

    def set_kernel(self, kind):
        check(lib().asg_plan_set_kernel(self._handle, int(kind)))

    def device_status(self):
        """Synchronise and raise AsgError if a kernel of this plan reported a bounded-wait timeout."""
        st = C.c_int(0)
        check(lib().asg_plan_device_status(self._handle, C.byref(st)))
        return st.value

    def update_ops(self, term_mats):
        mats = _as_term_mats(term_mats)
        ptrs = (C.POINTER(C.c_double) * (self.T * self.D))()
        lds = (C.c_int * (self.T * self.D))()
        for t in range(self.T):
            for d in range(self.D):
                ptrs[t * self.D + d] = mats[t][d].ctypes.data_as(C.POINTER(C.c_double))
                lds[t * self.D + d] = mats[t][d].shape[0]
        check(lib().asg_plan_update_ops(self._handle, ptrs, lds))
        self.term_mats = mats
        self._keep[0] = mats

    def apply(self, f, y=None, stream=None):
        """Device apply on CUDA tensors (float64 or float32); returns y."""
        import torch

        if not (f.is_cuda and f.is_contiguous() and f.numel() == self.dof_in):
            raise ValueError("f must be a contiguous CUDA tensor with %d values" % self.dof_in)
        if y is None:
            y = torch.empty(self.dof, dtype=f.dtype, device=f.device)
        if y.dtype != f.dtype or not y.is_cuda or y.numel() != self.dof or not y.is_contiguous():
            raise ValueError("y must be a contiguous CUDA tensor of f's type with %d values" % self.dof)
        s = stream if stream is not None else torch.cuda.current_stream(f.device)
        sp = C.c_void_p(s.cuda_stream)
        if f.dtype == torch.float64:
            check(lib().asg_apply_f64(self._handle, C.c_void_p(f.data_ptr()), C.c_void_p(y.data_ptr()), sp))
        elif f.dtype == torch.float32:
            check(lib().asg_apply_f32(self._handle, C.c_void_p(f.data_ptr()), C.c_void_p(y.data_ptr()), sp))
        else:
            raise TypeError("f must be float64 or float32")
        return y

    def apply_residual(self, f, ystar, r=None, stream=None):
        """r = A f - ystar (CUDA tensors of one type, three distinct buffers)."""
        import torch

        if not (f.is_cuda and f.is_contiguous() and f.numel() == self.dof_in):
            raise ValueError("f must be a contiguous CUDA tensor with %d values" % self.dof_in)
        if not (ystar.is_cuda and ystar.is_contiguous() and ystar.numel() == self.dof and ystar.dtype == f.dtype):
            raise ValueError("ystar must be a contiguous CUDA tensor of f's type with %d values" % self.dof)
        if r is None:
            r = torch.empty_like(ystar)
        if r.dtype != f.dtype or not r.is_cuda or r.numel() != self.dof or not r.is_contiguous():
            raise ValueError("r must be a contiguous CUDA tensor of f's type with %d values" % self.dof)
        s = stream if stream is not None else torch.cuda.current_stream(f.device)
        if f.dtype == torch.float64:
            fn = lib().asg_apply_residual_f64
        elif f.dtype == torch.float32:
            fn = lib().asg_apply_residual_f32
        else:
            raise TypeError("apply_residual supports float32 and float64")
        check(fn(self._handle, C.c_void_p(f.data_ptr()), C.c_void_p(ystar.data_ptr()), C.c_void_p(r.data_ptr()),
                 C.c_void_p(s.cuda_stream)))
        return r

    def apply_T(self, ybar, fbar=None, stream=None):
        """Adjoint on CUDA tensors: fbar = A^T ybar."""
        import torch

        if not (ybar.is_cuda and ybar.is_contiguous() and ybar.numel() == self.dof):
            raise ValueError("ybar must be a contiguous CUDA tensor with %d values" % self.dof)
        if fbar is None:
            fbar = torch.empty_like(ybar)
        s = stream if stream is not None else torch.cuda.current_stream(ybar.device)
        fn = lib().asg_apply_T_f64 if ybar.dtype == torch.float64 else lib().asg_apply_T_f32
        check(fn(self._handle, C.c_void_p(ybar.data_ptr()), C.c_void_p(fbar.data_ptr()), C.c_void_p(s.cuda_stream)))
        return fbar

    def grad_ops(self, f, r, stream=None):
        """dL/dA_{t,k} for every applied factor given y = A f and r = dL/dy (CUDA tensors).

        Returns T lists of d dense (n x n) column-major tensors (as [n, n] torch tensors in
        row-major view of the transposed storage, i.e. G[t][k][row, col]); identity factors the
        structure analysis skipped get None."""
        import torch

        T, D = self.T, self.D
        outs = [[None] * D for _ in range(T)]
        ptrs = (C.c_void_p * (T * D))()
        lds = (C.c_int * (T * D))()
        keep = []
        for t in range(T):
            for d in range(D):
                n = self.term_mats[t][d].shape[0]
                g = torch.zeros(n * n, dtype=f.dtype, device=f.device)
                keep.append(g)
                ptrs[t * D + d] = g.data_ptr()
                lds[t * D + d] = n
                outs[t][d] = g
        s = stream if stream is not None else torch.cuda.current_stream(f.device)
        fn = lib().asg_grad_ops_f64 if f.dtype == torch.float64 else lib().asg_grad_ops_f32
        check(fn(self._handle, C.c_void_p(f.data_ptr()), C.c_void_p(r.data_ptr()), ptrs, lds,
                 C.c_void_p(s.cuda_stream)))
        active = self.active_factors()
        res = []
        for t in range(T):
            row = []
            for d in range(D):
                n = self.term_mats[t][d].shape[0]
                row.append(outs[t][d].view(n, n).t() if active[t][d] else None)
            res.append(row)
        return res

    def active_factors(self):
        """[t][d] True where the plan applies operator (t, d) (False: a detected identity)."""
        masks = (C.c_uint * self.T)()
        check(lib().asg_plan_active(self._handle, masks))
        return [[bool((masks[t] >> d) & 1) for d in range(self.D)] for t in range(self.T)]

    def apply_host(self, f, out=None):
        """Host apply (copies in/out inside the library); numpy float64 or float32."""
        f = np.ascontiguousarray(f)
        if f.size != self.dof_in:
            raise ValueError("f must hold %d values" % self.dof_in)
        if out is None:
            out = np.empty(self.dof, dtype=f.dtype)
        if out.size != self.dof or out.dtype != f.dtype or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous array of f's type with %d values" % self.dof)
        if f.dtype == np.float64:
            check(lib().asg_apply_host_f64(self._handle, f.ctypes.data, out.ctypes.data))
        elif f.dtype == np.float32:
            check(lib().asg_apply_host_f32(self._handle, f.ctypes.data, out.ctypes.data))
        else:
            raise TypeError("f must be float64 or float32")
        return out

    def assemble_bsr(self, device=None):
        """The operator the plan applies as a scipy.sparse.bsr_matrix (FP64), assembled on the GPU
        (asg_assemble_bsr_f64; apply_A.m's build_A branch, apply_A.m:170-180,246-248)."""
        import scipy.sparse as sp
        import torch

        nb = C.c_longlong(0)
        check(lib().asg_assemble_bsr_f64(self._handle, None, None, None, 0, C.byref(nb), None))
        rp = np.zeros(self.N + 1, dtype=np.int64)
        cols = np.zeros(max(1, nb.value), dtype=np.int32)
        check(lib().asg_assemble_bsr_f64(self._handle, rp.ctypes.data_as(C.POINTER(C.c_longlong)),
                                         cols.ctypes.data_as(C.POINTER(C.c_int)), None, 0, C.byref(nb), None))
        dev = device if device is not None else torch.device("cuda", torch.cuda.current_device())
        blocks = torch.empty((max(1, nb.value), self.B, self.B), dtype=torch.float64, device=dev)
        check(lib().asg_assemble_bsr_f64(self._handle, None, None, C.c_void_p(blocks.data_ptr()), nb.value,
                                         C.byref(nb), C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)))
        data = blocks[:nb.value].cpu().numpy()
        return sp.bsr_matrix((data, cols[:nb.value], rp), shape=(self.dof, self.dof))

    def close(self):
        if self._handle:
            lib().asg_plan_destroy(self._handle)
            self._handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# -------------------------------------------------------------------------------------
# MATLAB-signature mirror: [ftmp, A, ALHS] = apply_A(pde, opts, A_data, f, deg, Vmax, Emax, imex_flag)
# -------------------------------------------------------------------------------------
_PLAN_CACHE = {}


def clear_plan_cache():
    for p in _PLAN_CACHE.values():
        p.close()
    _PLAN_CACHE.clear()


def _get(obj, name, default=None):
    if isinstance(obj, dict):
        return obj.get(name, default)
    return getattr(obj, name, default)


def _cached_plan(mats, idx, deg, pairs):
    key = (tuple((id(m), m.shape) for row in mats for m in row), idx.tobytes(), int(deg),
           None if pairs is None else (pairs[0].tobytes(), pairs[1].tobytes()))
    plan = _PLAN_CACHE.get(key)
    if plan is None:
        plan = Plan.create(mats, idx, deg, pairs=pairs, structure="detect", index_base=1)
        _PLAN_CACHE[key] = plan
    return plan


def apply_A(pde, opts, A_data, f, deg, Vmax=None, Emax=None, imex_flag="N", nargout=1):
    """Mirror of apply_A.m:1-252: returns ftmp = A*f as float64 numpy, or with nargout 2 or 3
    the tuple (ftmp, A, ALHS) of the reference's build_A branch.

    pde.terms[t].terms_1D[d].mat and pde.terms[t].imex select the terms (apply_A.m:19-28);
    opts.use_connectivity selects pde.connectivity (1-based lists) over all pairs
    (apply_A.m:44-52).  A is the operator of those terms over those pairs, assembled on the
    GPU (apply_A.m:170-180), a scipy sparse matrix when opts.use_sparse_A and a dense array
    otherwise; ALHS is the same assembly of pde.termsLHS, the non-identity LHS mass terms
    (apply_A.m:209-221), or 0 when there are none (apply_A.m:55).  Plans are cached per
    operator/index set like a MEX persistent handle; call clear_plan_cache() after mutating
    operators in place."""
    idx = np.stack([np.asarray(v).reshape(-1) for v in _get(A_data, "element_local_index_D")], axis=1)
    pairs = None
    if _get(opts, "use_connectivity", False):
        conn = _get(pde, "connectivity")
        lens = np.array([len(c) for c in conn], dtype=np.int64)
        rp = np.concatenate([[0], np.cumsum(lens)]).astype(np.int64)
        cl = np.concatenate([np.asarray(c, dtype=np.int64).reshape(-1) for c in conn]).astype(np.int32)
        pairs = (rp, cl)
    sparse = bool(_get(opts, "use_sparse_A", False))

    def assembled(terms):
        mats = [[_get(sd, "mat") for sd in _get(t, "terms_1D")] for t in terms]
        A = _cached_plan(mats, idx, deg, pairs).assemble_bsr()
        return A.tocsr() if sparse else A.toarray()

    terms = [t for t in _get(pde, "terms") if _get(t, "imex", "N") == imex_flag]
    n = np.asarray(f).size
    if terms:
        mats = [[_get(sd, "mat") for sd in _get(t, "terms_1D")] for t in terms]
        ftmp = _cached_plan(mats, idx, deg, pairs).apply_host(np.asarray(f, dtype=np.float64).reshape(-1))
    else:
        ftmp = np.zeros(n)
    if nargout <= 1:
        return ftmp
    if terms:
        A = assembled(terms)
    else:
        import scipy.sparse as sp

        A = sp.csr_matrix((n, n)) if sparse else np.zeros((n, n))
    lhs = _get(pde, "termsLHS") or []
    ALHS = assembled(lhs) if len(lhs) > 0 else 0
    return ftmp, A, ALHS


# -------------------------------------------------------------------------------------
# torch.autograd harness: y = A(ops) f with gradients for f and the 1-D operators
# -------------------------------------------------------------------------------------
def autograd_apply(plan, f, op_tensors=None):
    """y = A f through the plan with autograd support.

    ``op_tensors`` (optional) is a T x d nested list of torch tensors holding the plan's 1-D
    operators; gradients flow into those of them that require grad (the plan must have been
    created from the same values).  The backward pass runs the adjoint kernel for f and the
    deterministic operator-gradient kernel for the operators."""
    import torch

    flat = [] if op_tensors is None else [x for row in op_tensors for x in row]
    return _ApplyA.apply(plan, f, *flat)


def _make_function():
    import torch

    class ApplyA(torch.autograd.Function):
        @staticmethod
        def forward(ctx, plan, f, *ops):
            ctx.plan = plan
            ctx.nops = len(ops)
            ctx.save_for_backward(f)
            return plan.apply(f.contiguous())

        @staticmethod
        def backward(ctx, ybar):
            plan = ctx.plan
            (f,) = ctx.saved_tensors
            ybar = ybar.contiguous()
            fbar = plan.apply_T(ybar) if ctx.needs_input_grad[1] else None
            grads = [None] * ctx.nops
            if ctx.nops and any(ctx.needs_input_grad[2:]):
                G = plan.grad_ops(f, ybar)
                k = 0
                for t in range(plan.T):
                    for d in range(plan.D):
                        if ctx.needs_input_grad[2 + k]:
                            g = G[t][d]
                            n = plan.term_mats[t][d].shape[0]
                            grads[k] = g.contiguous() if g is not None else torch.zeros(n, n, dtype=f.dtype,
                                                                                        device=f.device)
                        k += 1
            return (None, fbar, *grads)

    return ApplyA


class _Lazy:
    fn = None

    @classmethod
    def apply(cls, *a):
        if cls.fn is None:
            cls.fn = _make_function()
        return cls.fn.apply(*a)


_ApplyA = _Lazy
