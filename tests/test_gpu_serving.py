"""Continuous batching on the GPU: every run's result is the same alone and in the mix.

Requests of different cases and sizes are served together: runs of one case and grid
share a bucket and advance with one batched graph launch per k steps (every kernel
covering all of the bucket's runs), buckets overlap on their own streams, and new runs
join while others are in flight. Each run is then stepped alone, eagerly, through the
one-run path. The final fields must be identical: runs share no data, each run's
pressure solves stop on their own, reductions are deterministic, and graph replay
equals eager stepping bit for bit.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def test_results_identical_alone_and_in_the_mix():
    from nyles_gb300 import serving as S
    from nyles_gb300.nyles import Nyles
    reqs = [S.Request(0, "lock", 32, 11, 20, 0.0), S.Request(1, "tgv", 16, 12, 20, 0.0),
            S.Request(2, "tgv", 48, 13, 10, 0.0), S.Request(3, "lock", 16, 14, 30, 0.0),
            S.Request(4, "lock", 32, 15, 20, 0.0)]
    # initial states built inline: all five are admitted in the loop's first pass
    eng = S.ServingEngine(precision="mixed", prep_threads=0)
    results, mixed_states = eng.serve(reqs, realtime=False, keep_states=True)
    assert eng.max_active == len(reqs)
    assert eng.buckets_made == 4                       # the two lock 32^3 runs share a bucket
    assert all(r.status == "ok" for r in results)
    # the same run alone in its bucket
    alone = S.ServingEngine(precision="mixed")
    _, alone_states = alone.serve([reqs[0]], realtime=False, keep_states=True)
    for s, arr in alone_states[0].items():
        np.testing.assert_array_equal(mixed_states[0][s], arr, err_msg="alone vs mix, field %s" % s)
    for req in reqs:
        nyl = Nyles(S.build_params(req.case, req.n, "mixed"))
        S.initial_state(nyl, req.case, req.seed)
        m = nyl.model
        m.diagnose_var(m.state)
        for _ in range(req.steps):
            m.forward(0.0, S.CASES[req.case]["dt"])
        for s, arr in mixed_states[req.rid].items():
            np.testing.assert_array_equal(m.state.get(s).view("i").double().cpu().numpy(), arr,
                                          err_msg="run %d field %s" % (req.rid, s))


def test_realtime_stream_latencies():
    from nyles_gb300 import serving as S
    reqs = S.make_requests(12, 40.0, seed=3, steps=10, sizes=(16, 32))
    eng = S.ServingEngine(precision="mixed")
    results, _ = eng.serve(reqs, realtime=True)
    assert len(results) == 12
    assert all(r.done >= r.admitted >= r.arrival - 1e-6 for r in results)
    s = S.summarize(results)
    assert 0 < s["p50_s"] <= s["p99_s"]


@pytest.mark.parametrize("case,n,precision", [("lock", 32, "mixed"), ("tgv", 48, "mixed"), ("lock", 32, "fp64")])
def test_footprint_model_covers_the_allocation(case, n, precision):
    """The admission footprint covers the arena of one run (state, registers, workspace)
    with at most 50% to spare, and a one-slot mixed bucket allocates about that much."""
    import gc
    from nyles_gb300 import serving as S
    from nyles_gb300.nyles import arena_bytes
    exact = arena_bytes(S.build_params(case, n, precision))
    need = S.footprint_bytes(case, n, precision)
    assert exact <= need <= 1.5 * exact, (exact, need)
    if precision == "mixed":
        gc.collect()
        torch.cuda.synchronize()
        before = torch.cuda.memory_allocated()
        b = S.Bucket((case, n, 10), precision, 1e-6, torch.device("cuda", torch.cuda.current_device()), 1)
        torch.cuda.synchronize()
        used = torch.cuda.memory_allocated() - before
        assert used <= need + (1 << 20), (used, need)
        b.close()
        del b


def test_batched_launches_are_fewer_than_per_run_launches():
    """A bucket of 6 runs of 32^3 is projected with one launch and advances its 30
    steps with one more (graph_steps): the library's kernel count for the ensemble is
    about one run's, not six. (Initial states built inline, so that all six are admitted in the first
    pass of the loop; with host threads they join as their states are ready.)"""
    from nyles_gb300 import _native as nat
    from nyles_gb300 import serving as S
    reqs = [S.Request(i, "tgv", 32, 20 + i, 30, 0.0) for i in range(6)]
    l0 = nat.lib().nyles_launch_count()
    eng = S.ServingEngine(precision="mixed", prep_threads=0)
    results, _ = eng.serve(reqs, realtime=False)
    batched = nat.lib().nyles_launch_count() - l0
    assert eng.launches == 2 and all(r.status == "ok" for r in results)   # one projection, one of 30 steps
    l0 = nat.lib().nyles_launch_count()
    one = S.ServingEngine(precision="mixed")
    one.serve(reqs[:1], realtime=False)
    single = nat.lib().nyles_launch_count() - l0
    assert batched < 1.5 * single, (batched, single)


def test_sequential_estimate_tracks_the_sequential_run():
    """The bucketed baseline (setup + steps x measured step time, queue replayed) stays
    within a factor of two of actually running the same requests one at a time."""
    from nyles_gb300 import serving as S
    reqs = [S.Request(0, "lock", 48, 11, 40, 0.0), S.Request(1, "tgv", 32, 12, 40, 0.0),
            S.Request(2, "lock", 48, 13, 40, 0.0)]
    est, timing = S.sequential_estimate(reqs, precision="fp64", sample_steps=10)
    run, _ = S.run_sequential(reqs, precision="fp64")
    assert set(timing) == {("lock", 48), ("tgv", 32)}
    span_est = max(r.done for r in est)
    span_run = max(r.done for r in run)
    assert 0.5 < span_est / span_run < 2.0, (span_est, span_run)
