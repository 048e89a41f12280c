"""Mirror of the reference's Kronecker entry points on the GPU (Kronmult/, kron_multd.m, krond.m).

* ``KronPlan``        kronmultN_batch.m's per-level GEMM lists for kron(A1..An)*X, executed
                      on the device one batched launch per level.
* ``kron_multd``      Y = kron_multd(nkron, Acell, X) (kron_multd.m:1) through a KronPlan.
* ``kronmult_batch``  [batch_lists..., Y] = kronmultN_batch(A1..An, X, lists...) (Kronmult/
                      kronmult{1..6}_batch.m:1-3): returns the lists as dictionaries with the
                      reference's fields and Y.
* ``gemm_vbatched``   Clist = gemm_vbatched(transA, transB, mlist, nlist, klist, alpha, Alist,
                      Blist, beta, Clist) (Kronmult/gemm_vbatched.m:1), k from klist.
* ``krond``           Y = krond(nkron, Acell) (krond.m:1).

Matrices are column-major (numpy arrays are converted); torch is used only for device memory.
"""
import ctypes as C

import numpy as np

from ._lib import GemmDesc, check, lib


def _dev(a, dtype):
    import torch

    t = torch.from_numpy(np.asfortranarray(a, dtype=dtype).reshape(-1, order="F").copy())
    return t.cuda()


class KronPlan:
    """kron(A1..An) * X for fixed factor shapes and nvec columns."""

    def __init__(self, shapes, nvec):
        self.shapes = [(int(r), int(c)) for r, c in shapes]
        self.n = len(self.shapes)
        self.nvec = int(nvec)
        nr = (C.c_int * self.n)(*[r for r, _ in self.shapes])
        nc = (C.c_int * self.n)(*[c for _, c in self.shapes])
        self._h = C.c_void_p()
        check(lib().asg_kron_plan_create(self.n, nr, nc, self.nvec, C.byref(self._h)))
        b64, b32 = C.c_size_t(0), C.c_size_t(0)
        check(lib().asg_kron_plan_workspace(self._h, C.byref(b64), C.byref(b32)))
        self.work_bytes = {8: b64.value, 4: b32.value}
        self.rows = int(np.prod([r for r, _ in self.shapes]))
        self.cols = int(np.prod([c for _, c in self.shapes]))

    def lists(self):
        """The recorded GEMM descriptors (host), one dict per GEMM, in execution order."""
        cnt = C.c_int(0)
        check(lib().asg_kron_plan_lists(self._h, None, 0, C.byref(cnt)))
        arr = (GemmDesc * max(1, cnt.value))()
        check(lib().asg_kron_plan_lists(self._h, arr, cnt.value, C.byref(cnt)))
        out = []
        for d in arr[:cnt.value]:
            out.append({k: (getattr(d, k).decode() if k.startswith("trans") else getattr(d, k)) for k, _ in GemmDesc._fields_})
        return out

    def apply(self, A_dev, X_dev, Y_dev=None, work=None, stream=None):
        """Device execution: A_dev list of CUDA tensors (column-major flattened), X_dev [cols*nvec]."""
        import torch

        dt = X_dev.dtype
        es = 8 if dt == torch.float64 else 4
        if Y_dev is None:
            Y_dev = torch.empty(self.rows * self.nvec, dtype=dt, device=X_dev.device)
        if work is None:
            work = torch.empty(max(1, self.work_bytes[es] // es), dtype=dt, device=X_dev.device)
        ptrs = (C.c_void_p * self.n)(*[a.data_ptr() for a in A_dev])
        s = stream if stream is not None else torch.cuda.current_stream(X_dev.device)
        fn = lib().asg_kron_batch_f64 if es == 8 else lib().asg_kron_batch_f32
        check(fn(self._h, ptrs, C.c_void_p(X_dev.data_ptr()), C.c_void_p(Y_dev.data_ptr()), C.c_void_p(work.data_ptr()),
                 work.numel() * es, C.c_void_p(s.cuda_stream)))
        return Y_dev

    def close(self):
        if self._h:
            lib().asg_kron_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def kron_multd(nkron, Acell, X):
    """Y = kron(A{1},...,A{nkron}) * X with X holding prod(ncols) x nvec values (kron_multd.m)."""
    import torch

    mats = [np.asarray(a, dtype=np.float64) for a in Acell[:nkron]]
    if len(mats) < nkron:
        raise ValueError("kron_multd: invalid nkron=%d, length(Acell)=%d" % (nkron, len(Acell)))
    cols = int(np.prod([m.shape[1] for m in mats]))
    X = np.asarray(X, dtype=np.float64)
    if X.size % cols:
        raise ValueError("kron_multd:nkron=%d,prod(size(X))=%g,isizeX=%g" % (nkron, X.size, cols))
    nvec = X.size // cols
    plan = KronPlan([m.shape for m in mats], nvec)
    Ad = [_dev(m, np.float64) for m in mats]
    Y = plan.apply(Ad, _dev(X.reshape(cols, nvec, order="F"), np.float64))
    torch.cuda.synchronize()
    out = Y.cpu().numpy().reshape(plan.rows, nvec, order="F")
    plan.close()
    return out


def kronmult_batch(mats, X):
    """(lists, Y): lists[L] holds the GEMMs kronmult{n}_batch appends to batch_list{L+1}, each a
    dict with m, n, k, transA, transB, alpha, beta and the operand values A, B, C (C after the
    product); Y = kron(A1..An) * X."""
    import torch

    mats = [np.asarray(a, dtype=np.float64) for a in mats]
    n = len(mats)
    cols = int(np.prod([m.shape[1] for m in mats]))
    X = np.asarray(X, dtype=np.float64)
    nvec = X.size // cols
    plan = KronPlan([m.shape for m in mats], nvec)
    Ad = [_dev(m, np.float64) for m in mats]
    Xd = _dev(X.reshape(cols, nvec, order="F"), np.float64)
    work = torch.zeros(max(1, plan.work_bytes[8] // 8), dtype=torch.float64, device="cuda")
    Yd = plan.apply(Ad, Xd, work=work)
    torch.cuda.synchronize()
    bufs = [a.cpu().numpy() for a in Ad] + [Xd.cpu().numpy(), Yd.cpu().numpy()]
    wk = work.cpu().numpy()
    descs = plan.lists()
    lists = [[] for _ in range(n)]
    srcs = bufs + [wk]  # operand ids: factors, X, Y, workspace

    def operand(op, off, rows, cols_, ld):
        idx = off + np.arange(cols_)[None, :] * ld + np.arange(rows)[:, None]
        return srcs[op][idx]

    for d in descs:
        ta, tb = d["trans_a"], d["trans_b"]
        ar, ac = (d["k"], d["m"]) if ta in "Tt" else (d["m"], d["k"])
        br, bc = (d["n"], d["k"]) if tb in "Tt" else (d["k"], d["n"])
        lists[d["level"] - 1].append({
            "m": d["m"], "n": d["n"], "k": d["k"], "transA": ta, "transB": tb, "alpha": d["alpha"], "beta": d["beta"],
            "A": operand(d["a_operand"], d["a_offset"], ar, ac, d["lda"]),
            "B": operand(d["b_operand"], d["b_offset"], br, bc, d["ldb"]),
            "C": operand(d["c_operand"], d["c_offset"], d["m"], d["n"], d["ldc"]),
        })
    Y = bufs[n + 1].reshape(plan.rows, nvec, order="F")
    plan.close()
    return lists, Y


def gemm_vbatched(transA, transB, mlist, nlist, klist, alpha, Alist, Blist, beta, Clist):
    """Kronmult/gemm_vbatched.m on the GPU: returns the list of C matrices."""
    import torch

    nb = len(mlist)
    if not (len(nlist) == nb and len(klist) == nb and len(Alist) == nb and len(Blist) == nb and len(Clist) == nb):
        raise ValueError("gemm_vbatched: mismatch nbatch=%d" % nb)
    dA = [_dev(a, np.float64) for a in Alist]
    dB = [_dev(b, np.float64) for b in Blist]
    dC = [_dev(c, np.float64) for c in Clist]
    ld = lambda arrs: torch.tensor([np.asarray(a).shape[0] for a in arrs], dtype=torch.int32, device="cuda")
    ptr = lambda ts: torch.tensor([t.data_ptr() for t in ts], dtype=torch.int64, device="cuda")
    m = torch.tensor(list(mlist), dtype=torch.int32, device="cuda")
    n = torch.tensor(list(nlist), dtype=torch.int32, device="cuda")
    k = torch.tensor(list(klist), dtype=torch.int32, device="cuda")
    pA, pB, pC = ptr(dA), ptr(dB), ptr(dC)
    lA, lB, lC = ld(Alist), ld(Blist), ld(Clist)
    s = torch.cuda.current_stream()
    check(lib().asg_gemm_vbatched_f64(transA.encode(), transB.encode(), m.data_ptr(), n.data_ptr(), k.data_ptr(),
                                      float(alpha), pA.data_ptr(), lA.data_ptr(), pB.data_ptr(), lB.data_ptr(),
                                      float(beta), pC.data_ptr(), lC.data_ptr(), nb, C.c_void_p(s.cuda_stream)))
    torch.cuda.synchronize()
    return [c.cpu().numpy().reshape(np.asarray(c0).shape, order="F") for c, c0 in zip(dC, Clist)]


def krond(nkron, Acell):
    """kron(A{1}, kron(A{2}, ...)) on the GPU (krond.m)."""
    import torch

    mats = [np.asarray(a, dtype=np.float64) for a in Acell[:nkron]]
    nr = (C.c_int * nkron)(*[m.shape[0] for m in mats])
    nc = (C.c_int * nkron)(*[m.shape[1] for m in mats])
    rows = int(np.prod([m.shape[0] for m in mats]))
    cols = int(np.prod([m.shape[1] for m in mats]))
    dA = [_dev(m, np.float64) for m in mats]
    out = torch.empty(rows * cols, dtype=torch.float64, device="cuda")
    ptrs = (C.c_void_p * nkron)(*[a.data_ptr() for a in dA])
    check(lib().asg_krond_f64(nkron, nr, nc, ptrs, C.c_void_p(out.data_ptr()),
                              C.c_void_p(torch.cuda.current_stream().cuda_stream)))
    torch.cuda.synchronize()
    return out.cpu().numpy().reshape(rows, cols, order="F")
