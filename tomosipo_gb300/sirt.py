"""SIRT on the GB300 projector: the reference recipe, and a batched multi-job solver.

The recipe (``README.md:150-163``, ``doc/intro/fast_reconstruction.rst:92-104``)::

    R = min(1 / A(1), 1 / ts.epsilon)        # per ray
    C = min(1 / A.T(1), 1 / ts.epsilon)      # per voxel
    x += C * A.T(R * (y - A(x)))             # per iteration

``sirt`` runs it exactly like that with the operator and torch element-wise
ops ("looping the plain operator"). ``BatchedSirt`` runs one iteration of many
independent jobs (any mix of sizes and geometries) as a handful of kernel
launches over all jobs, with the residual ``R * (y - A x)`` fused into the
forward projector's epilogue and ``x += C * A.T(r)`` into the backprojector's;
an iteration can be captured in a CUDA graph. Both produce the same numbers:
the fused epilogues use the same operations in the same order, without FMA
contraction.
"""
import ctypes

import torch

from . import _native

EPSILON = 1e-8  # ts.epsilon (tomosipo/__init__.py:41)


def preconditioners(A, device):
    """R (sinogram-shaped) and C (volume-shaped), clipped at 1 / epsilon."""
    R = A(torch.ones(A.domain_shape, device=device))
    torch.reciprocal(R, out=R)
    torch.clamp(R, max=1 / EPSILON, out=R)
    C = A.T(torch.ones(A.range_shape, device=device))
    torch.reciprocal(C, out=C)
    torch.clamp(C, max=1 / EPSILON, out=C)
    return R, C


def sirt(A, y, num_iterations=10, x_init=None, R=None, C=None):
    """Reference SIRT: ``num_iterations`` of ``x += C * A.T(R * (y - A(x)))``."""
    dev = y.device
    if R is None or C is None:
        R, C = preconditioners(A, dev)
    x = torch.zeros(A.domain_shape, device=dev) if x_init is None else x_init.clone()
    y_tmp = torch.empty(A.range_shape, device=dev)
    x_tmp = torch.empty(A.domain_shape, device=dev)
    for _ in range(num_iterations):
        A(x, out=y_tmp)
        torch.sub(y, y_tmp, out=y_tmp)
        y_tmp.mul_(R)
        A.T(y_tmp, out=x_tmp)
        x_tmp.mul_(C)
        x.add_(x_tmp)
    return x


class BatchedSirt:
    """SIRT for many independent jobs, advanced together.

    ``jobs`` is a list of ``(A, y)`` or ``(A, y, x_init)`` with ``y`` a CUDA
    tensor on one device; jobs may differ in size and geometry (their
    detectors' v axis must run along z: circular and helical scans). Each
    iteration is three kernel launches over all jobs. ``run(n, graph=True)``
    captures one iteration in a CUDA graph and replays it. ``x[i]`` is job i's
    reconstruction, equal to ``sirt(A_i, y_i, n)``.
    """

    def __init__(self, jobs):
        if not jobs:
            raise ValueError("BatchedSirt needs at least one job")
        self.device = jobs[0][1].device
        if self.device.type != "cuda":
            raise ValueError("BatchedSirt runs on CUDA tensors")
        lib = _native.load()
        self._keep = []
        self.x, self.R, self.C = [], [], []
        table = (_native.SirtJob * len(jobs))()
        with torch.cuda.device(self.device):
            for i, job in enumerate(jobs):
                A, y = job[0], job[1]
                x0 = job[2] if len(job) > 2 else None
                if y.device != self.device:
                    raise ValueError("all jobs must be on the same device")
                y = y.to(torch.float32).contiguous()
                R, C = preconditioners(A, self.device)
                x = (torch.zeros(A.domain_shape, device=self.device) if x0 is None
                     else x0.to(self.device, torch.float32).contiguous().clone())
                res = torch.empty(A.range_shape, device=self.device)
                nbytes = A.projector.workspace_bytes(self.device.index, True)
                ws = torch.empty(max(nbytes, 4) // 4, device=self.device)
                self._keep += [A, y, res, ws]
                self.x.append(x)
                self.R.append(R)
                self.C.append(C)
                t = table[i]
                t.projector = A.projector.handle(self.device.index)
                t.vol, t.sino, t.R, t.C = x.data_ptr(), y.data_ptr(), R.data_ptr(), C.data_ptr()
                t.residual, t.fp_workspace = res.data_ptr(), ws.data_ptr()
            out = ctypes.c_void_p()
            _native.check(lib.tsgb_sirt_batch_create(table, len(jobs), ctypes.byref(out)),
                          "tsgb_sirt_batch_create")
        self._batch = out.value
        self._graph = None

    def step(self, iterations=1):
        """Queue ``iterations`` iterations on the current stream."""
        lib = _native.load()
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device).cuda_stream
            _native.check(lib.tsgb_sirt_batch_iterate(self._batch, int(iterations), stream),
                          "tsgb_sirt_batch_iterate")

    def _capture(self):
        g = torch.cuda.CUDAGraph()
        with torch.cuda.device(self.device):
            with torch.cuda.graph(g):
                self.step(1)
        return g

    def run(self, num_iterations, graph=True):
        """Run ``num_iterations`` iterations (graph replays if ``graph``)."""
        if not graph:
            self.step(num_iterations)
            return self.x
        if self._graph is None:
            self._graph = self._capture()
        for _ in range(num_iterations):
            self._graph.replay()
        return self.x

    def close(self):
        if getattr(self, "_batch", None):
            _native.load().tsgb_sirt_batch_destroy(self._batch)
            self._batch = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
