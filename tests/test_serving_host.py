"""Host logic of the serving engine on the CPU: request stream, footprint model,
admission against the HBM budget, completion bookkeeping (fake runs, no GPU)."""
import numpy as np

from nyles_gb300 import serving as S


def test_request_stream_is_seeded_poisson():
    a = S.make_requests(96, 20.0, seed=5, steps=300)
    b = S.make_requests(96, 20.0, seed=5, steps=300)
    assert [(r.case, r.n, r.seed, r.arrival) for r in a] == [(r.case, r.n, r.seed, r.arrival) for r in b]
    gaps = np.diff([0.0] + [r.arrival for r in a])
    assert 0.03 < gaps.mean() < 0.08          # 1/20 s on average
    assert {r.n for r in a} <= {32, 48, 64, 96, 128} and {r.case for r in a} == {"lock", "tgv"}


def test_footprint_grows_with_size_and_precision():
    f = [S.footprint_bytes("tgv", n, "mixed") for n in (32, 48, 64, 96, 128)]
    assert all(x < y for x, y in zip(f, f[1:]))
    assert S.footprint_bytes("lock", 64, "fp64") > 1.5 * S.footprint_bytes("lock", 64, "mixed")
    assert S.steps_per_graph(300) == 10 and S.steps_per_graph(7) == 7 and S.steps_per_graph(13) == 1


class FakeRun:
    """Stands in for a resident run: each launch completes on the next poll."""
    live = 0
    peak = 0

    def __init__(self, req, precision, device, mg_tol, priority=0):
        self.req = req
        self.priority = priority
        self.k = S.steps_per_graph(req.steps)
        self.launched = 0
        self.pending = 0
        FakeRun.live += 1
        FakeRun.peak = max(FakeRun.peak, FakeRun.live)

    def launch(self):
        self.launched += self.k
        self.pending += 1

    def poll(self):
        n = self.pending
        self.pending = 0
        return n

    @property
    def all_launched(self):
        return self.launched >= self.req.steps

    def finished(self):
        done = self.all_launched and self.poll() == 0
        if done:
            FakeRun.live -= 1
        return done

    # rid -> status reported at completion (default "ok")
    outcomes = {}

    def outcome(self):
        return FakeRun.outcomes.get(self.req.rid, "ok"), 0

    def final_state(self):
        return {}


def test_admission_respects_the_budget_and_serves_everything():
    FakeRun.live = FakeRun.peak = 0
    reqs = S.make_requests(20, 20.0, seed=1, steps=30, sizes=(64,))
    one = S.footprint_bytes("lock", 64, "mixed")
    eng = S.ServingEngine(hbm_budget_bytes=3.5 * one, device="cpu", run_factory=FakeRun)
    results, _ = eng.serve(reqs, realtime=False)
    assert [r.rid for r in results] == list(range(20))
    assert eng.max_active <= 3 and eng.peak_used <= 3.5 * one
    assert FakeRun.live == 0
    summary = S.summarize(results)
    assert summary["runs"] == 20 and summary["p99_s"] >= summary["p50_s"]


def test_replay_queue_one_at_a_time():
    """The sequential baseline's queue: starts at max(arrival, previous end)."""
    from nyles_gb300 import serving as S
    reqs = [S.Request(0, "lock", 32, 1, 10, 0.0), S.Request(1, "tgv", 64, 2, 10, 0.5),
            S.Request(2, "lock", 32, 3, 10, 5.0)]
    res = S.replay_queue(reqs, lambda r: 1.0 if r.n == 32 else 2.0)
    assert [(r.rid, r.admitted, r.done) for r in res] == [(0, 0.0, 1.0), (1, 1.0, 3.0), (2, 5.0, 6.0)]
    assert [r.latency for r in res] == [1.0, 2.5, 1.0]


def test_stream_priorities_by_work():
    """Smallest work gets the greatest (numerically lowest) priority; equal work, equal
    priority; "none" leaves every stream at 0."""
    from nyles_gb300 import serving as S
    reqs = [S.Request(i, "lock", n, i, 300, 0.0) for i, n in enumerate((32, 48, 64, 96, 128, 32))]
    eng = S.ServingEngine(device="cpu", run_factory=FakeRun)
    pr = eng.stream_priorities(reqs, levels=(0, -5))
    assert pr[0] == pr[5] == -5 and pr[4] > pr[3] > pr[2] > pr[1] > pr[0] and pr[4] <= 0
    assert set(S.ServingEngine(device="cpu", run_factory=FakeRun, priority="none")
               .stream_priorities(reqs).values()) == {0}


def test_window_serves_shortest_remaining_work_first():
    """With a window of one run and every request available at once, runs complete in
    the order of their work; every run completes."""
    from nyles_gb300 import serving as S
    sizes = [96, 32, 128, 48, 64]
    reqs = [S.Request(i, "lock", n, i, 20, 0.0) for i, n in enumerate(sizes)]
    ticks = iter(range(10 ** 6))
    eng = S.ServingEngine(device="cpu", run_factory=FakeRun, window=1, clock=lambda: float(next(ticks)))
    results, _ = eng.serve(reqs, realtime=False)
    order = [r.rid for r in sorted(results, key=lambda r: r.done)]
    assert order == sorted(range(5), key=lambda i: sizes[i])
    assert FakeRun.live == 0


def test_oversize_request_refused_while_the_others_finish():
    """A request whose footprint exceeds the whole budget is refused at once (it could
    never be admitted); the others are served and release their memory; a run that blew
    up is counted, not timed."""
    FakeRun.live = FakeRun.peak = 0
    FakeRun.outcomes = {3: "blowup"}
    try:
        reqs = [S.Request(i, "lock", 64, i, 20, 0.01 * i) for i in range(6)]
        reqs[2] = S.Request(2, "tgv", 128, 2, 20, 0.02)
        budget = 2.5 * S.footprint_bytes("lock", 64, "mixed")
        assert S.footprint_bytes("tgv", 128, "mixed") > budget
        eng = S.ServingEngine(hbm_budget_bytes=budget, device="cpu", run_factory=FakeRun)
        results, _ = eng.serve(reqs, realtime=False)
    finally:
        FakeRun.outcomes = {}
    status = {r.rid: r.status for r in results}
    assert status == {0: "ok", 1: "ok", 2: "refused", 3: "blowup", 4: "ok", 5: "ok"}
    assert eng.used == 0 and FakeRun.live == 0 and eng.peak_used <= budget
    summary = S.summarize(results)
    assert summary["runs"] == 4 and summary["refused"] == 1 and summary["blowup"] == 1
