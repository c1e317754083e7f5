"""SIRT on the GB300 projector: the reference recipe, and a batched multi-job solver.

The recipe (``README.md:150-163``, ``doc/intro/fast_reconstruction.rst:92-104``)::

    R = min(1 / A(1), 1 / ts.epsilon)        # per ray
    C = min(1 / A.T(1), 1 / ts.epsilon)      # per voxel
    x += C * A.T(R * (y - A(x)))             # per iteration

``sirt`` runs it exactly like that with the operator and torch element-wise
ops ("looping the plain operator"). ``BatchedSirt`` advances many independent
jobs (any mix of sizes and geometries) together: per job and iteration one
forward kernel whose epilogue writes the residual ``W R (y - A x)`` and one
backward kernel whose epilogue applies ``x += C A.T(r)``, with jobs spread
over concurrent streams and iterations captured in a CUDA graph. Both produce
the same numbers: the fused epilogues use the same operations in the same
order, without FMA contraction.
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


class SirtJobState:
    """Device buffers of one SIRT job: x, y, R, C, residual and FP workspace."""

    def __init__(self, A, y, x_init=None, device=None):
        device = y.device if device is None else device
        if device.type != "cuda":
            raise ValueError("batched SIRT runs on CUDA tensors")
        self.A = A
        self.device = device
        with torch.cuda.device(device):
            self.y = y.to(device=device, dtype=torch.float32).contiguous()
            self.R, self.C = preconditioners(A, device)
            self.x = (torch.zeros(A.domain_shape, device=device) if x_init is None
                      else x_init.to(device, torch.float32).contiguous().clone())
            rows, angles, cols = A.range_shape
            # the backprojector's row-pair layout (two floats per pixel) with two
            # zero detector rows above and below, read as padding
            self.res = torch.zeros(2 * (rows + 4) * angles * cols, device=device)
            nbytes = A.projector.workspace_bytes(device.index, True)
            self.ws = torch.empty(max(nbytes, 4) // 4, device=device)

    def tensors(self):
        return (self.y, self.R, self.C, self.x, self.res, self.ws)

    @staticmethod
    def device_bytes(A):
        """Device memory a job holds: x, C (volume) and y, R, residual (sinogram) plus workspace."""
        vol = 4 * int(torch.Size(A.domain_shape).numel())
        rows, angles, cols = A.range_shape
        sino = 4 * rows * angles * cols
        stats_ws = A.projector.stats(torch.cuda.current_device())["fp_workspace_bytes"]
        return 2 * vol + 4 * sino + 32 * angles * cols + stats_ws


def make_states(jobs, device, n_streams=4):
    """SirtJobState of each ``(A, y)`` or ``(A, y, x_init)``, built on up to
    ``n_streams`` side streams at once (each job's preconditioners are one
    forward and one backprojection, too small alone to fill the GPU); the
    current stream waits for all of them. The results do not depend on the
    stream a job's setup ran on."""
    main = torch.cuda.current_stream(device)
    if len(jobs) < 2:
        return [SirtJobState(j[0], j[1], j[2] if len(j) > 2 else None, device) for j in jobs]
    side = [torch.cuda.Stream(device) for _ in range(min(n_streams, len(jobs)))]
    for s in side:
        s.wait_stream(main)  # the inputs are written on the current stream
    states = []
    for i, j in enumerate(jobs):
        with torch.cuda.stream(side[i % len(side)]):
            st = SirtJobState(j[0], j[1], j[2] if len(j) > 2 else None, device)
        for t in st.tensors():
            t.record_stream(main)  # used from now on on the current stream
        states.append(st)
    for s in side:
        main.wait_stream(s)
    return states


def autotune_jobs(operators, device):
    """Autotune the forward schedules of many operators: one autotuner run per
    (volume shape, detector shape, beam kind), its schedule set on every
    operator of that shape (the batch launches each job's forward projection in
    its projector's schedule). Returns {shape key: tuning}."""
    from .autotune import autotune, shape_key

    tuning = {}
    with torch.cuda.device(device):
        for A in operators:
            key = shape_key(A.projector)
            if key not in tuning:
                tuning[key] = autotune(A, device.index, key=key)["tuning"]
            A.projector.set_tuning(device.index, **tuning[key])
    return tuning


class NativeBatch:
    """Native job table over a list of SirtJobState (rebuilt when jobs change)."""

    def __init__(self, states):
        if not states:
            raise ValueError("a batch needs at least one job")
        self.states = list(states)
        self.device = states[0].device
        lib = _native.load()
        table = (_native.SirtJob * len(states))()
        for i, st in enumerate(states):
            if st.device != self.device:
                raise ValueError("all jobs must be on the same device")
            t = table[i]
            t.projector = st.A.projector.handle(self.device.index)
            t.vol, t.sino, t.R, t.C = st.x.data_ptr(), st.y.data_ptr(), st.R.data_ptr(), st.C.data_ptr()
            t.residual, t.fp_workspace = st.res.data_ptr(), st.ws.data_ptr()
        out = ctypes.c_void_p()
        with torch.cuda.device(self.device):
            _native.check(lib.tsgb_sirt_batch_create(table, len(states), ctypes.byref(out)),
                          "tsgb_sirt_batch_create")
        self._batch = out.value

    def step(self, iterations=1):
        lib = _native.load()
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device).cuda_stream
            _native.check(lib.tsgb_sirt_batch_iterate(self._batch, int(iterations), stream),
                          "tsgb_sirt_batch_iterate")

    def step_jobs(self, iterations):
        """``iterations[i]`` iterations of job i (creation order) on the current stream."""
        lib = _native.load()
        counts = (ctypes.c_int32 * len(self.states))(*[int(k) for k in iterations])
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device).cuda_stream
            _native.check(lib.tsgb_sirt_batch_iterate_jobs(self._batch, counts, stream),
                          "tsgb_sirt_batch_iterate_jobs")

    def close(self):
        if getattr(self, "_batch", None):
            _native.load().tsgb_sirt_batch_destroy(self._batch)
            self._batch = None

    def __del__(self):
        try:
            self.close()
        except Exception:  # a finalizer: at interpreter exit the library may be gone
            pass


class BatchedSirt:
    """SIRT for many independent jobs, advanced together.

    ``jobs`` is a list of ``(A, y)`` or ``(A, y, x_init)`` with ``y`` a CUDA
    tensor on one device; jobs may differ in size and geometry (their
    detectors' v axis must run along z: circular and helical scans). With
    ``autotune`` the forward schedules come from the autotuner, one run per
    job shape (``tomosipo_gb300.autotune``; results are cached per shape).
    ``run(n, graph=True)`` captures ``graph_iterations`` iterations of all jobs
    in one CUDA graph (a job's next iteration need not wait for the other
    jobs) and replays it. ``x[i]`` is job i's reconstruction, equal to
    ``sirt(A_i, y_i, n)``.
    """

    graph_iterations = 10

    def __init__(self, jobs, autotune=False):
        if not jobs:
            raise ValueError("BatchedSirt needs at least one job")
        self.device = jobs[0][1].device
        if self.device.type != "cuda":
            raise ValueError("BatchedSirt runs on CUDA tensors")
        self.tuning = autotune_jobs([j[0] for j in jobs], self.device) if autotune else {}
        with torch.cuda.device(self.device):
            self.states = make_states(jobs, self.device)
        self._native = NativeBatch(self.states)
        self._graphs = {}

    @property
    def x(self):
        return [st.x for st in self.states]

    @property
    def R(self):
        return [st.R for st in self.states]

    @property
    def C(self):
        return [st.C for st in self.states]

    def step(self, iterations=1):
        """Queue ``iterations`` iterations on the current stream."""
        self._native.step(iterations)

    def _graph(self, iterations):
        g = self._graphs.get(iterations)
        if g is None:
            g = torch.cuda.CUDAGraph()
            with torch.cuda.device(self.device):
                with torch.cuda.graph(g):
                    self.step(iterations)
            self._graphs[iterations] = g
        return g

    def run(self, num_iterations, graph=True):
        """Run ``num_iterations`` iterations (CUDA graph replays if ``graph``)."""
        if not graph:
            self.step(num_iterations)
            return self.x
        chunk = max(1, min(self.graph_iterations, num_iterations))
        full, rest = divmod(num_iterations, chunk)
        if full:
            g = self._graph(chunk)
            for _ in range(full):
                g.replay()
        if rest:
            self._graph(rest).replay()
        return self.x

    def close(self):
        self._native.close()
