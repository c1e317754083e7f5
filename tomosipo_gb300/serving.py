"""Continuous-batching SIRT server.

Requests (an operator, a measured sinogram and an iteration count) arrive over
time. The server admits waiting requests first-come-first-served while their
device memory fits the budget, advances admitted jobs with one batched launch
sequence per step (``NativeBatch``), and retires jobs as they finish, so
requests that arrive while others run join at the next step and their work
shares the device with the running jobs.

Which jobs a step advances is the scheduling policy. ``"srpt"`` (default):
each step has a work budget of one iteration of the largest active job; jobs
are taken in order of least remaining work (remaining iterations times the
per-iteration cost, voxels x angles) and each gets as many iterations as fit,
so small jobs finish in a few steps instead of waiting for the largest one
(shortest remaining processing time first, the order that minimises mean
latency); a job passed over for ``max_wait_steps`` steps gets one iteration
anyway. ``"all"``: every active job one iteration per step. Each job's
arithmetic is independent of the others and of the schedule, so a result is
the same alone, in any mix and under either policy.

There is no counterpart in the reference (its SIRT is a per-job Python loop,
``README.md:150-163``). Failure handling is host-side: requests larger than
the whole budget are rejected, a request whose set-up raises is marked failed
without disturbing the others, and requests can be cancelled while waiting or
running.
"""
import dataclasses
import math
import time
from collections import deque


@dataclasses.dataclass
class Request:
    id: int
    A: object                 # operator (its detector's v axis must run along z)
    y: object                 # measured sinogram (CUDA tensor)
    iterations: int = 20
    arrival: float = 0.0      # seconds after the server's start


@dataclasses.dataclass
class Result:
    id: int
    status: str               # "done", "rejected", "failed" or "cancelled"
    x: object = None
    arrival: float = 0.0
    admitted: float = math.nan
    finished: float = math.nan
    error: str = ""

    @property
    def latency(self):
        return self.finished - self.arrival


class GpuEngine:
    """Runs jobs with the batched SIRT kernels."""

    def job_bytes(self, req):
        from .sirt import SirtJobState

        return SirtJobState.device_bytes(req.A)

    def job_cost(self, req):
        """Work of one iteration (voxels x angles; FP + BP scale with it)."""
        n_vox = 1
        for d in req.A.domain_shape:
            n_vox *= int(d)
        return float(n_vox * req.A.range_shape[1])

    def admit(self, req):
        from .sirt import SirtJobState

        return SirtJobState(req.A, req.y)

    def build(self, states):
        from .sirt import NativeBatch

        return NativeBatch(states)

    def step(self, batch, iterations):
        import torch

        batch.step_jobs(iterations)
        torch.cuda.synchronize(batch.device)

    def result(self, state):
        return state.x

    def release(self, batch):
        if batch is not None:
            batch.close()


class _Active:
    __slots__ = ("req", "state", "remaining", "bytes", "admitted", "cost", "waited")

    def __init__(self, req, state, nbytes, admitted, cost):
        self.req = req
        self.state = state
        self.remaining = req.iterations
        self.bytes = nbytes
        self.admitted = admitted
        self.cost = cost        # work of one iteration
        self.waited = 0         # consecutive steps without an iteration


class SirtServer:
    """First-come-first-served admission by memory; SRPT (or all-jobs) steps."""

    def __init__(self, engine=None, memory_budget=None, max_active=64, memory_fraction=0.8,
                 policy="srpt", max_wait_steps=4):
        if policy not in ("srpt", "all"):
            raise ValueError(f"policy must be 'srpt' or 'all'. Got {policy!r}")
        self.policy = policy
        self.max_wait_steps = int(max_wait_steps)
        self.engine = engine if engine is not None else GpuEngine()
        if memory_budget is None:
            import torch

            free, _total = torch.cuda.mem_get_info()
            memory_budget = int(free * memory_fraction)
        self.memory_budget = int(memory_budget)
        self.max_active = int(max_active)
        self.used = 0
        self.steps = 0
        self.max_concurrent = 0
        self._cancelled = set()

    def plan_step(self, active):
        """Iterations each active job runs in the next step (``active`` order)."""
        if self.policy == "all":
            return [1] * len(active)
        left = max(j.cost for j in active)
        order = sorted(range(len(active)),
                       key=lambda i: (active[i].remaining * active[i].cost, active[i].req.arrival,
                                      active[i].req.id))
        iters = [0] * len(active)
        for rank, i in enumerate(order):
            j = active[i]
            k = max(0, min(j.remaining, int(left // j.cost))) if j.cost > 0 else j.remaining
            if k == 0 and (rank == 0 or j.waited >= self.max_wait_steps):
                k = 1
            iters[i] = k
            left -= k * j.cost
        return iters

    def cancel(self, req_id):
        """Cancel a waiting or running request (takes effect at the next step)."""
        self._cancelled.add(req_id)

    def run(self, requests, clock=None, sleep=None):
        """Serve ``requests`` (arrival times relative to the call) to completion.

        Returns one Result per request, in request order.
        """
        clock = clock or time.perf_counter
        sleep = sleep or time.sleep
        t0 = clock()
        now = lambda: clock() - t0  # noqa: E731
        pending = deque(sorted(requests, key=lambda r: (r.arrival, r.id)))
        waiting = deque()
        active = []
        results = {r.id: Result(r.id, "pending", arrival=r.arrival) for r in requests}
        batch = None
        changed = False

        def retire(job, status, x=None):
            nonlocal changed
            res = results[job.req.id]
            res.status = status
            res.x = x
            res.finished = now()
            self.used -= job.bytes
            active.remove(job)
            changed = True

        while pending or waiting or active:
            t = now()
            while pending and pending[0].arrival <= t:
                waiting.append(pending.popleft())
            # cancellations
            for req in [r for r in waiting if r.id in self._cancelled]:
                waiting.remove(req)
                results[req.id].status = "cancelled"
                results[req.id].finished = now()
            for job in [j for j in active if j.req.id in self._cancelled]:
                retire(job, "cancelled")
            # admission, first come first served
            while waiting and len(active) < self.max_active:
                req = waiting[0]
                try:
                    need = int(self.engine.job_bytes(req))
                except Exception as e:  # bad request: fail it, keep serving
                    waiting.popleft()
                    results[req.id].status, results[req.id].error = "failed", repr(e)
                    results[req.id].finished = now()
                    continue
                if need > self.memory_budget:
                    waiting.popleft()
                    results[req.id].status = "rejected"
                    results[req.id].error = (
                        f"needs {need} bytes, more than the {self.memory_budget}-byte budget")
                    results[req.id].finished = now()
                    continue
                if self.used + need > self.memory_budget:
                    break  # wait for running jobs to free memory
                waiting.popleft()
                try:
                    state = self.engine.admit(req)
                except Exception as e:
                    results[req.id].status, results[req.id].error = "failed", repr(e)
                    results[req.id].finished = now()
                    continue
                self.used += need
                job = _Active(req, state, need, now(), float(self.engine.job_cost(req)))
                results[req.id].admitted = job.admitted
                active.append(job)
                changed = True
            if not active:
                if pending and not waiting:
                    sleep(max(0.0, min(pending[0].arrival - now(), 0.05)))
                elif waiting:
                    # nothing fits and nothing runs: the head request can never start
                    req = waiting.popleft()
                    results[req.id].status = "rejected"
                    results[req.id].error = "cannot be admitted"
                    results[req.id].finished = now()
                continue
            if changed:
                self.engine.release(batch)
                batch = self.engine.build([j.state for j in active])
                changed = False
            self.max_concurrent = max(self.max_concurrent, len(active))
            iters = self.plan_step(active)
            self.engine.step(batch, iters)
            self.steps += 1
            for job, k in zip(list(active), iters):
                job.remaining -= k
                job.waited = 0 if k else job.waited + 1
                if job.remaining <= 0:
                    retire(job, "done", self.engine.result(job.state))
        self.engine.release(batch)
        return [results[r.id] for r in requests]


def _percentile(values, p):
    v = sorted(values)
    k = (len(v) - 1) * p
    lo, hi = math.floor(k), math.ceil(k)
    return v[lo] + (v[hi] - v[lo]) * (k - lo)


def latency_stats(results):
    """Latency of the completed requests (s): end to end (p50 / p99), split into
    queueing (arrival to admission) and service (admission to completion);
    throughput (solves/s over the span from the first arrival to the last
    completion) and request counts."""
    done = [r for r in results if r.status == "done"]
    if not done:
        return {"completed": 0, "n_requests": len(results)}
    lat = [r.latency for r in done]
    queue = [r.admitted - r.arrival for r in done]
    service = [r.finished - r.admitted for r in done]
    span = max(r.finished for r in done) - min(r.arrival for r in done)
    return {
        "n_requests": len(results),
        "completed": len(done),
        "p50_s": _percentile(lat, 0.50),
        "p99_s": _percentile(lat, 0.99),
        "queue_p50_s": _percentile(queue, 0.50),
        "queue_p99_s": _percentile(queue, 0.99),
        "service_p50_s": _percentile(service, 0.50),
        "service_p99_s": _percentile(service, 0.99),
        "solves_per_s": len(done) / span if span > 0 else math.inf,
    }
