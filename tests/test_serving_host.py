"""Host logic of the serving engine on the CPU: request stream, footprint model,
admission against the HBM budget, buckets and completion bookkeeping (fake buckets, no
GPU)."""
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
    assert S.footprint_bytes("lock", 64, "fp64") > 1.4 * S.footprint_bytes("lock", 64, "mixed")
    assert S.steps_per_graph(300) == 10 and S.steps_per_graph(7) == 7 and S.steps_per_graph(13) == 1
    assert S.graph_steps(128, 300) == 10 and S.graph_steps(32, 300) == 60 and S.graph_steps(64, 300) == 60
    assert S.graph_steps(96, 300) == 20 and S.graph_steps(32, 7) == 7


class FakeSlot:
    def __init__(self, index):
        self.index = index
        self.req = None
        self.launched = 0
        self.admitted = 0.0
        self.pending = 0

    @property
    def active(self):
        return self.req is not None and self.launched < self.req.steps

    def finished(self):
        return self.req is not None and self.launched >= self.req.steps and self.pending == 0


class FakeBucket:
    """Stands in for a bucket of resident runs: each launch advances every active slot
    by k steps and completes on the next poll."""
    live = 0
    peak = 0
    made = []
    # rid -> status reported at completion (default "ok")
    outcomes = {}

    def __init__(self, key, precision, mg_tol, device, capacity, priority=0):
        self.key = key
        self.case, self.n, self.k = key
        self.capacity = capacity
        self.bytes = capacity * S.footprint_bytes(self.case, self.n, precision)
        self.slots = [FakeSlot(r) for r in range(capacity)]
        self.launches = 0
        self.priority = priority
        FakeBucket.made.append(self)

    def free_slot(self):
        return next((sl for sl in self.slots if sl.req is None), None)

    def resident(self):
        return [sl for sl in self.slots if sl.req is not None]

    def admit(self, slot, req, now, staged=None):
        slot.req, slot.launched, slot.admitted, slot.pending = req, 0, now, 0
        FakeBucket.live += 1
        FakeBucket.peak = max(FakeBucket.peak, FakeBucket.live)

    def poll(self):
        for sl in self.slots:
            sl.pending = 0
        return 0

    def launch(self):
        act = [sl for sl in self.slots if sl.active]
        for sl in act:
            sl.launched += self.k
            sl.pending = 1
        self.launches += bool(act)
        return bool(act)

    def outcome(self, slot, keep_state=False):
        return FakeBucket.outcomes.get(slot.req.rid, "ok"), 0, None

    def release(self, slot):
        slot.req = None
        FakeBucket.live -= 1

    def close(self):
        pass


def _reset():
    FakeBucket.live = FakeBucket.peak = 0
    FakeBucket.made = []
    FakeBucket.outcomes = {}


def test_admission_respects_the_budget_and_serves_everything():
    _reset()
    reqs = S.make_requests(20, 20.0, seed=1, steps=30, sizes=(64,))
    one = S.footprint_bytes("lock", 64, "mixed")
    eng = S.ServingEngine(hbm_budget_bytes=3.5 * one, device="cpu", bucket_factory=FakeBucket)
    results, _ = eng.serve(reqs, realtime=False)
    assert [r.rid for r in results] == list(range(20))
    assert all(r.status == "ok" for r in results)
    assert eng.max_active <= 3 and eng.peak_used <= 3.5 * one
    assert FakeBucket.live == 0
    summary = S.summarize(results)
    assert summary["runs"] == 20 and summary["p99_s"] >= summary["p50_s"]


def test_runs_of_a_bucket_share_its_launches():
    """Runs of the same case and grid sit in one bucket and advance together: the
    launches are far fewer than one per run and step group."""
    _reset()
    reqs = [S.Request(i, "tgv", 32, i, 30, 0.0) for i in range(8)] + [S.Request(8, "lock", 32, 8, 30, 0.0)]
    eng = S.ServingEngine(device="cpu", bucket_factory=FakeBucket, capacity=16)
    results, _ = eng.serve(reqs, realtime=False)
    assert len(results) == 9 and eng.buckets_made == 2
    assert eng.launches == 2 * 1           # 30 steps of 32^3 in one launch, once per bucket
    assert eng.max_active == 9


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
    eng = S.ServingEngine(device="cpu", bucket_factory=FakeBucket)
    pr = eng.stream_priorities(reqs, levels=(0, -5))
    assert pr[0] == pr[5] == -5 and pr[4] > pr[3] > pr[2] > pr[1] > pr[0] and pr[4] <= 0
    assert set(S.ServingEngine(device="cpu", bucket_factory=FakeBucket, priority="none")
               .stream_priorities(reqs).values()) == {0}


def test_oversize_request_refused_while_the_others_finish():
    """A request whose footprint exceeds the whole budget is refused at once (it could
    never be admitted); the others are served and release their memory; a run that blew
    up is counted, not timed."""
    _reset()
    FakeBucket.outcomes = {3: "blowup"}
    reqs = [S.Request(i, "lock", 64, i, 20, 0.01 * i) for i in range(6)]
    reqs[2] = S.Request(2, "tgv", 128, 2, 20, 0.02)
    budget = 2.5 * S.footprint_bytes("lock", 64, "mixed")
    assert S.footprint_bytes("tgv", 128, "mixed") > budget
    eng = S.ServingEngine(hbm_budget_bytes=budget, device="cpu", bucket_factory=FakeBucket)
    results, _ = eng.serve(reqs, realtime=False)
    status = {r.rid: r.status for r in results}
    assert status == {0: "ok", 1: "ok", 2: "refused", 3: "blowup", 4: "ok", 5: "ok"}
    assert eng.used == 0 and FakeBucket.live == 0 and eng.peak_used <= budget
    summary = S.summarize(results)
    assert summary["runs"] == 4 and summary["refused"] == 1 and summary["blowup"] == 1
