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

    def __init__(self, req, precision, device, mg_tol):
        self.req = req
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

    def vcycles(self):
        return 0

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
