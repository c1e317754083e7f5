"""Continuous-batching SIRT server.

Requests (an operator, a measured sinogram and an iteration count) arrive over
time. The server admits waiting requests first-come-first-served while their
device memory fits the budget, advances every admitted job by one SIRT
iteration per step with one batched launch sequence (``NativeBatch``), and
retires jobs as they finish, so requests that arrive while others run join at
the next step and their work shares the device with the running jobs. Each
job's arithmetic is independent of the others in the batch, so a result is
the same alone and in any mix.

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

    def admit(self, req):
        from .sirt import SirtJobState

        return SirtJobState(req.A, req.y)

    def build(self, states):
        from .sirt import NativeBatch

        return NativeBatch(states)

    def step(self, batch):
        import torch

        batch.step(1)
        torch.cuda.synchronize(batch.device)

    def result(self, state):
        return state.x

    def release(self, batch):
        if batch is not None:
            batch.close()


class _Active:
    __slots__ = ("req", "state", "remaining", "bytes", "admitted")

    def __init__(self, req, state, nbytes, admitted):
        self.req = req
        self.state = state
        self.remaining = req.iterations
        self.bytes = nbytes
        self.admitted = admitted


class SirtServer:
    """First-come-first-served admission by memory; one iteration per step."""

    def __init__(self, engine=None, memory_budget=None, max_active=64, memory_fraction=0.8):
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
                job = _Active(req, state, need, now())
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
            self.engine.step(batch)
            self.steps += 1
            for job in list(active):
                job.remaining -= 1
                if job.remaining <= 0:
                    retire(job, "done", self.engine.result(job.state))
        self.engine.release(batch)
        return [results[r.id] for r in requests]


def latency_stats(results):
    """p50 / p99 latency (s) and throughput (solves/s) of the completed requests."""
    done = [r for r in results if r.status == "done"]
    if not done:
        return {"completed": 0}
    lat = sorted(r.latency for r in done)

    def pct(p):
        k = (len(lat) - 1) * p
        lo, hi = math.floor(k), math.ceil(k)
        return lat[lo] + (lat[hi] - lat[lo]) * (k - lo)

    span = max(r.finished for r in done) - min(r.arrival for r in done)
    return {
        "completed": len(done),
        "p50_s": pct(0.50),
        "p99_s": pct(0.99),
        "solves_per_s": len(done) / span if span > 0 else math.inf,
    }
