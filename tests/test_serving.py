"""Host logic of the continuous-batching SIRT server, with a fake engine and a
fake clock (CPU): admission by memory, joining mid-run, rejection, failure
isolation, cancellation and latency statistics."""
import pytest

from tomosipo_gb300.serving import Request, SirtServer, latency_stats


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t

    def sleep(self, dt):
        self.t += max(dt, 1e-3)


class FakeEngine:
    """Each step takes `step_time`; a job's state counts its iterations."""

    def __init__(self, clock, sizes, step_time=1.0, fail_ids=(), costs=None):
        self.clock, self.sizes, self.step_time = clock, sizes, step_time
        self.fail_ids = set(fail_ids)
        self.costs = costs or {}
        self.batches = []
        self.steps = []

    def job_bytes(self, req):
        return self.sizes[req.id]

    def job_cost(self, req):
        return self.costs.get(req.id, 1.0)

    def admit(self, req):
        if req.id in self.fail_ids:
            raise RuntimeError("geometry not supported")
        return {"id": req.id, "iters": 0}

    def build(self, states):
        self.batches.append(sorted(s["id"] for s in states))
        return list(states)

    def step(self, batch, iterations):
        self.steps.append({s["id"]: k for s, k in zip(batch, iterations)})
        for s, k in zip(batch, iterations):
            s["iters"] += k
        # with per-job costs a step takes as long as the work it runs
        work = sum(k * self.costs.get(s["id"], 1.0) for s, k in zip(batch, iterations))
        self.clock.t += self.step_time * (max(1.0, work) if self.costs else 1.0)

    def result(self, state):
        return state["iters"]

    def release(self, batch):
        pass


def _server(sizes, budget, **kw):
    clock = FakeClock()
    eng = FakeEngine(clock, sizes,
                     **{k: v for k, v in kw.items() if k in ("step_time", "fail_ids", "costs")})
    srv = SirtServer(engine=eng, memory_budget=budget, max_active=kw.get("max_active", 64),
                     policy=kw.get("policy", "all"))
    return clock, eng, srv


def test_all_jobs_complete_with_their_iterations():
    clock, eng, srv = _server({0: 10, 1: 10, 2: 10}, 100)
    reqs = [Request(i, None, None, iterations=3 + i, arrival=0.0) for i in range(3)]
    res = srv.run(reqs, clock=clock, sleep=clock.sleep)
    assert [r.status for r in res] == ["done"] * 3
    assert [r.x for r in res] == [3, 4, 5]
    assert srv.max_concurrent == 3


def test_admission_waits_for_memory_and_joins_mid_run():
    # budget fits two jobs; job 2 waits until one finishes, then joins the running job
    clock, eng, srv = _server({0: 40, 1: 40, 2: 40}, 100)
    reqs = [Request(0, None, None, 2, 0.0), Request(1, None, None, 5, 0.0), Request(2, None, None, 2, 0.0)]
    res = srv.run(reqs, clock=clock, sleep=clock.sleep)
    assert all(r.status == "done" for r in res)
    assert eng.batches[0] == [0, 1]
    assert [1, 2] in eng.batches  # continuous batching: 2 runs alongside 1
    assert res[2].admitted >= res[0].finished
    assert res[2].x == 2


def test_late_arrival_joins_running_batch():
    clock, eng, srv = _server({0: 10, 1: 10}, 100)
    reqs = [Request(0, None, None, 10, 0.0), Request(1, None, None, 3, 2.5)]
    res = srv.run(reqs, clock=clock, sleep=clock.sleep)
    assert eng.batches == [[0], [0, 1], [0]]
    assert res[1].admitted < res[0].finished
    assert res[1].latency == pytest.approx(res[1].finished - 2.5)


def test_oversized_request_is_rejected_others_served():
    clock, eng, srv = _server({0: 500, 1: 10}, 100)
    res = srv.run([Request(0, None, None, 2, 0.0), Request(1, None, None, 2, 0.0)],
                  clock=clock, sleep=clock.sleep)
    assert res[0].status == "rejected" and "budget" in res[0].error
    assert res[1].status == "done"


def test_failed_setup_is_isolated():
    clock, eng, srv = _server({0: 10, 1: 10, 2: 10}, 100, fail_ids={1})
    res = srv.run([Request(i, None, None, 2, 0.0) for i in range(3)], clock=clock, sleep=clock.sleep)
    assert [r.status for r in res] == ["done", "failed", "done"]
    assert "geometry" in res[1].error
    assert srv.used == 0


def test_cancellation_of_waiting_and_running():
    clock, eng, srv = _server({0: 60, 1: 60, 2: 10}, 100)
    srv.cancel(1)
    reqs = [Request(0, None, None, 4, 0.0), Request(1, None, None, 4, 0.0), Request(2, None, None, 4, 0.0)]
    res = srv.run(reqs, clock=clock, sleep=clock.sleep)
    assert [r.status for r in res] == ["done", "cancelled", "done"]
    clock2, eng2, srv2 = _server({0: 10}, 100)

    class CancelMidway(FakeEngine):
        def step(self, batch, iterations):
            super().step(batch, iterations)
            if batch[0]["iters"] == 2:
                srv2.cancel(0)

    eng2.__class__ = CancelMidway
    res2 = srv2.run([Request(0, None, None, 10, 0.0)], clock=clock2, sleep=clock2.sleep)
    assert res2[0].status == "cancelled" and srv2.used == 0


def test_latency_stats():
    clock, eng, srv = _server({i: 1 for i in range(10)}, 100, max_active=2)
    reqs = [Request(i, None, None, 1, 0.0) for i in range(10)]
    st = latency_stats(srv.run(reqs, clock=clock, sleep=clock.sleep))
    assert st["completed"] == 10
    assert st["p50_s"] == pytest.approx(3.0, abs=0.6)
    assert st["p99_s"] == pytest.approx(5.0, abs=0.1)
    assert st["solves_per_s"] == pytest.approx(2.0)
    # two run at a time, one step (1 s) each: queueing grows with the backlog,
    # service stays one step; latency = queueing + service for every request
    assert st["n_requests"] == 10
    assert st["service_p50_s"] == pytest.approx(1.0, abs=0.05)
    assert st["service_p99_s"] == pytest.approx(1.0, abs=0.05)
    assert st["queue_p50_s"] == pytest.approx(st["p50_s"] - 1.0, abs=0.6)
    assert st["queue_p99_s"] == pytest.approx(4.0, abs=0.1)


def test_srpt_finishes_small_jobs_first_with_the_same_results():
    # one large job (cost 8 per iteration) and three small ones (cost 1), 10 iterations each
    costs = {0: 8.0, 1: 1.0, 2: 1.0, 3: 1.0}
    reqs = [Request(i, None, None, iterations=10, arrival=0.0) for i in range(4)]
    out = {}
    for policy in ("all", "srpt"):
        clock, eng, srv = _server({i: 1 for i in range(4)}, 100, costs=costs, policy=policy)
        out[policy] = (srv.run(reqs, clock=clock, sleep=clock.sleep), eng)
    all_res, srpt_res = out["all"][0], out["srpt"][0]
    assert [r.x for r in srpt_res] == [r.x for r in all_res] == [10] * 4
    small_all = sorted(r.latency for r in all_res[1:])
    small_srpt = sorted(r.latency for r in srpt_res[1:])
    assert max(small_srpt) < min(small_all)  # every small job finishes earlier
    assert latency_stats(srpt_res)["p50_s"] < latency_stats(all_res)["p50_s"]
    # the large job is not starved: makespan within the total work plus the step granularity
    assert srpt_res[0].latency <= sum(10 * c for c in costs.values()) + 8


def test_srpt_plan_respects_budget_and_wait_limit():
    from tomosipo_gb300.serving import _Active

    srv = SirtServer(engine=FakeEngine(FakeClock(), {}), memory_budget=1, policy="srpt",
                     max_wait_steps=2)

    def job(i, remaining, cost, waited=0):
        j = _Active(Request(i, None, None, remaining, 0.0), None, 0, 0.0, cost)
        j.waited = waited
        return j

    big, small = job(0, 5, 4.0), job(1, 10, 1.0)
    assert srv.plan_step([big, small]) == [0, 4]          # budget 4: four small iterations
    assert srv.plan_step([job(0, 5, 4.0, waited=2), small]) == [1, 4]  # waited too long
    assert srv.plan_step([big]) == [1]
    assert srv.plan_step([job(0, 1, 4.0), job(1, 1, 1.0)]) == [0, 1]  # less remaining work first
    # a forced iteration overdraws the budget: later jobs get 0, never a negative count
    plan = srv.plan_step([job(0, 9, 4.0, waited=2), job(1, 3, 3.0, waited=0), job(2, 8, 4.0)])
    assert plan == [0, 1, 0] or min(plan) >= 0
    assert min(srv.plan_step([job(0, 2, 4.0), job(1, 9, 3.0, waited=3), job(2, 9, 4.0, waited=3)])) >= 0
