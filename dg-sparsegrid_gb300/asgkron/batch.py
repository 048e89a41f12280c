"""Many independent y_k = A_k f_k in one persistent launch (asg_batch_*), optionally captured
into a CUDA graph; across ranks the problems are sharded with no communication
(``partition_problems``)."""
import ctypes as C

from ._lib import check, lib


def partition_problems(costs, nparts):
    """Problem indices per rank, [[k, ...], ...]: longest-processing-time greedy (problems by
    descending cost, ties by index, each to the least-loaded rank, ties to the lowest rank).
    Every problem goes to exactly one rank and the largest load is at most the mean plus the
    largest single cost.  Each rank's list is in ascending problem order."""
    if nparts < 1:
        raise ValueError("partition_problems: nparts=%d" % nparts)
    costs = [float(c) for c in costs]
    if any(c < 0 for c in costs):
        raise ValueError("partition_problems: negative cost")
    load = [0.0] * nparts
    parts = [[] for _ in range(nparts)]
    for k in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        r = min(range(nparts), key=lambda j: (load[j], j))
        parts[r].append(k)
        load[r] += costs[k]
    return [sorted(p) for p in parts]


class Batch:
    def __init__(self, plans):
        self.plans = list(plans)
        arr = (C.c_void_p * len(self.plans))(*[p.handle for p in self.plans])
        self._h = C.c_void_p()
        check(lib().asg_batch_create(arr, len(self.plans), C.byref(self._h)))
        self.graph = None

    def set_io(self, fs, ys):
        """Device tensors per problem (all float64 or all float32); uploads the problem table."""
        import torch

        self._io = (list(fs), list(ys))
        fp = (C.c_void_p * len(fs))(*[f.data_ptr() for f in fs])
        yp = (C.c_void_p * len(ys))(*[y.data_ptr() for y in ys])
        self.precision = 0 if fs[0].dtype == torch.float64 else 1
        fn = lib().asg_batch_set_io_f64 if self.precision == 0 else lib().asg_batch_set_io_f32
        check(fn(self._h, fp, yp))
        check(lib().asg_batch_prepare(self._h, self.precision))

    def apply(self, stream=None):
        import torch

        s = stream if stream is not None else torch.cuda.current_stream()
        check(lib().asg_batch_apply(self._h, self.precision, C.c_void_p(s.cuda_stream)))

    def tune(self):
        import torch

        ms = C.c_float(0)
        check(lib().asg_batch_tune(self._h, self.precision, C.c_void_p(torch.cuda.current_stream().cuda_stream),
                                   C.byref(ms)))
        return ms.value

    def configure(self, warps_per_cta, rows_per_item):
        """Fixed launch shape instead of tune(): 4 or 8 warps per CTA, 1, 2 or 4 rows per item."""
        check(lib().asg_batch_configure(self._h, int(warps_per_cta), int(rows_per_item)))

    def info(self):
        w, r, fl = C.c_int(0), C.c_int(0), C.c_double(0)
        check(lib().asg_batch_info(self._h, C.byref(w), C.byref(r), C.byref(fl)))
        return {"warps_per_cta": w.value, "rows_per_item": r.value, "flops": fl.value}

    def capture(self):
        import torch

        self.apply()
        torch.cuda.synchronize()
        self.graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(self.graph):
            self.apply()
        return self.graph

    def close(self):
        if self._h:
            lib().asg_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
