"""Failure detection on the GPU, every failure made on the host (no device fault, trap
or hang): a NaN written into an initial state, a multigrid stop rule that cannot be
met, a captured graph whose solves stop at maxite, a serving request larger than the
whole HBM budget.

Each failure comes back as a status: NYLES_BLOWUP / BlowUp and the blow-up flag of
forward and Nyles.run (the reference's flag is never set), NYLES_NOT_CONVERGED and the
not_converged counters (core/mgfor/solvers.f90:8-33 stops at maxite without a word),
and the serving engine's "refused" result.
"""
import ctypes

import numpy as np
import pytest

import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


def _nyles(**cfg):
    from nyles_gb300.nyles import Nyles
    return Nyles(helpers.make_params(**cfg))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_nan_in_initial_buoyancy_stops_forward_and_run(precision):
    from nyles_gb300 import _native as nat
    cfg = dict(geometry="closed", n=(16, 16, 16), dt=1e-3, precision=precision, mg_tol=1e-12, mg_maxite=20)
    # forward: the NaN reaches the velocity through Bernoulli's buoyancy term in the first
    # stage, whose projection stops with NYLES_BLOWUP
    nyl = _nyles(**cfg)
    m = nyl.model
    b = np.zeros(tuple(m.state.b.view("i").shape))
    b[5, 6, 7] = np.nan
    m.state.b.view("i")[...] = torch.from_numpy(b)
    m.diagnose_var(m.state)                          # the projection sees a finite divergence
    assert m.forward(0.0, 1e-3) is True
    assert m.mg_stats()["nonfinite"] == 1
    assert b"non-finite" in nat.lib().nyles_last_error()
    # Nyles.run: stops after the first step and reports the blow-up
    nyl = _nyles(**cfg)
    nyl.model.state.b.view("i")[...] = torch.from_numpy(b)
    t, n, blowup = nyl.run(nsteps=5, verbose=False)
    assert blowup and n == 1


def test_nan_in_initial_velocity_raises_blowup():
    from nyles_gb300 import _native as nat
    nyl = _nyles(geometry="perio_xyz", n=(16, 16, 16), dt=1e-3)
    m = nyl.model
    u = np.zeros(tuple(m.state.u["i"].view("i").shape))
    u[4, 4, 4] = np.nan
    m.state.u["i"].view("i")[...] = torch.from_numpy(u)
    with pytest.raises(nat.BlowUp):
        m.diagnose_var(m.state)
    nyl = _nyles(geometry="perio_xyz", n=(16, 16, 16), dt=1e-3)
    nyl.model.state.u["i"].view("i")[...] = torch.from_numpy(u)
    t, n, blowup = nyl.run(nsteps=3, verbose=False)
    assert blowup and n == 0


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_standalone_solve_reports_not_converged(precision):
    """maxite = 1 at tol 1e-30: the C ABI returns NYLES_NOT_CONVERGED with the stats of
    the one V-cycle; a NaN right-hand side returns NYLES_BLOWUP at once."""
    from nyles_gb300 import _native as nat
    from nyles_gb300.multigrid import MG
    mg = MG(16, 16, 16, "closed", precision)
    rng = np.random.Generator(np.random.PCG64(3))
    b = rng.standard_normal((16, 16, 16))
    b -= b.mean()
    mg.set(1, 2, torch.from_numpy(b))
    mg.set_params(1e-30, 1, 0.9)
    st = nat.NylesMgStats()
    rc = nat.lib().nyles_mg_solve(mg._h, ctypes.byref(st), nat.stream_ptr())
    assert rc == nat.NYLES_NOT_CONVERGED
    assert st.nite == 1 and st.res > 1e-30 and st.not_converged == 1 and st.nonfinite == 0
    x, info = mg.solve()
    assert not info["converged"] and info["nite"] == 1
    b[1, 2, 3] = np.nan
    mg.set(1, 2, torch.from_numpy(b))
    mg.set_params(1e-6, 20, 0.9)
    rc = nat.lib().nyles_mg_solve(mg._h, ctypes.byref(st), nat.stream_ptr())
    assert rc == nat.NYLES_BLOWUP and st.nite == 0 and st.nonfinite == 1
    with pytest.raises(nat.BlowUp):
        mg.solve()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_graph_solves_stop_at_maxite_and_are_counted(precision):
    """A captured step whose pressure solves cannot reach tol (1e-30) runs exactly maxite
    V-cycles per solve on the device, returns, and counts every solve as not converged;
    the state stays finite and equal to eager stepping's."""
    cfg = dict(geometry="perio_xy", n=(16, 16, 32), L=(1.0, 1.0, 2.0), dt=1e-3, precision=precision,
               mg_tol=1e-30, mg_maxite=3)
    runs = []
    for graphs in (False, True):
        nyl = _nyles(**cfg)
        m = nyl.model
        m.use_graphs = graphs
        helpers.load_state(nyl, _NullOracle(), helpers.seeded_state(nyl, "noise", 7))
        m.diagnose_var(m.state)
        s0 = m.mg_stats()
        if graphs:
            m.capture_graph(1e-3, 2)
            m.replay()
        else:
            for _ in range(2):
                m.forward(0.0, 1e-3)
        torch.cuda.synchronize()
        s1 = m.mg_stats()
        assert s1["not_converged"] - s0["not_converged"] == 6    # 3 solves per RK3 step
        assert s1["vcycles"] - s0["vcycles"] == 18 and s1["nite"] == 3
        assert s1["nonfinite"] == 0
        runs.append({f: m.state.get(f).view("i").double().cpu().numpy() for f in ("b", "u_i", "p")})
    for f in ("b", "u_i", "p"):
        assert np.isfinite(runs[1][f]).all()
        assert np.array_equal(runs[0][f], runs[1][f]), f


def test_graph_solve_stops_on_nonfinite_norm():
    """A NaN reaching a replayed step's projections stops each solve's loop at once (no
    V-cycle) and is counted on the device; Nyles.run turns the count into its blow-up
    flag after a replayed step."""
    nyl = _nyles(geometry="closed", n=(16, 16, 16), dt=1e-3, mg_tol=1e-12, mg_maxite=20)
    m = nyl.model
    m.diagnose_var(m.state)
    m.capture_graph(1e-3, 1)
    b = np.zeros(tuple(m.state.b.view("i").shape))
    b[3, 3, 3] = np.nan
    m.state.b.view("i")[...] = torch.from_numpy(b)
    s0 = m.mg_stats()
    m.replay()
    torch.cuda.synchronize()
    s1 = m.mg_stats()
    # the NaN reaches the velocity in the first stage (Bernoulli's buoyancy term), so all
    # three projections of the step see a non-finite divergence
    assert s1["nonfinite"] - s0["nonfinite"] == 3
    assert s1["vcycles"] - s0["vcycles"] == 0
    # Nyles.run: the first two steps run eagerly (the graph is captured on the second
    # repeat of dt); a NaN written after two clean steps is caught after a replayed one
    nyl = _nyles(geometry="closed", n=(16, 16, 16), dt=1e-3, mg_tol=1e-12, mg_maxite=20)

    def poison(ny, t, n):
        if n == 3:
            ny.model.state.b.view("i")[3, 3, 3] = float("nan")

    t, n, blowup = nyl.run(nsteps=8, verbose=False, callback=poison)
    assert nyl.model.graph is not None
    assert blowup and n == 4


def test_serving_refuses_a_request_above_the_budget():
    """A request whose footprint exceeds the whole budget is refused while the others
    are served and release their memory."""
    from nyles_gb300 import serving as S
    reqs = [S.Request(0, "lock", 32, 11, 20, 0.0), S.Request(1, "tgv", 64, 12, 20, 0.0),
            S.Request(2, "lock", 32, 13, 20, 0.0)]
    budget = 1.5 * S.footprint_bytes("tgv", 32, "mixed")
    assert S.footprint_bytes("tgv", 64, "mixed") > budget
    free0 = torch.cuda.mem_get_info()[0]
    eng = S.ServingEngine(hbm_budget_bytes=budget, precision="mixed")
    results, _ = eng.serve(reqs, realtime=False)
    assert {r.rid: r.status for r in results} == {0: "ok", 1: "refused", 2: "ok"}
    assert eng.used == 0
    torch.cuda.empty_cache()
    assert torch.cuda.mem_get_info()[0] >= free0 - (64 << 20)


class _NullOracle:
    """load_state's oracle side, discarded: only the GPU state is needed here."""

    def field(self, name):
        return _Sink()


class _Sink:
    def __setitem__(self, key, value):
        pass
