"""CUDA-graph replay of time steps against eager stepping: identical bits.

The captured graph runs the same kernels in the same order; the multigrid stop test
moves to the device (a conditional while-node), so V-cycle counts and every field must
equal the eager path's exactly.
"""
import numpy as np
import pytest

import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = [
    (dict(geometry="closed", n=(32, 16, 16), L=(2.0, 1.0, 1.0), dt=2e-3), "lock", 1),
    (dict(geometry="perio_xy", n=(16, 16, 32), L=(1.0, 1.0, 2.0), n_tracers=1, dt=1e-3), "noise", 2),
    (dict(geometry="perio_xyz", n=(16, 16, 16), L=(6.283185307179586,) * 3, modelname="Euler3d",
          timestepping="LFAM3", dt=5e-3), "tgv", 1),
    (dict(geometry="perio_xy", n=(16, 16, 32), L=(1.0, 1.0, 2.0), dt=1e-3, precision="mixed",
          mg_tol=1e-20), "noise", 1),
    (dict(geometry="closed", n=(16, 16, 16), timestepping="EF", dt=1e-3, diff_coef={"u": 1e-3}), "noise", 3),
]


def _model(cfg, kind, seed, graphs=False):
    from nyles_gb300.nyles import Nyles
    nyl = Nyles(helpers.make_params(**cfg))
    nyl.model.use_graphs = graphs
    for k, v in helpers.seeded_state(nyl, kind, seed).items():
        nyl.model.state.get(k).view("i")[...] = torch.from_numpy(v)
    nyl.model.diagnose_var(nyl.model.state)
    return nyl


def _assert_same_state(a, b):
    for s in a.model.state.toc:
        for comp in (["i", "j", "k"] if a.model.state.toc[s] != "scalar" else [None]):
            name = s if comp is None else s + "_" + comp
            np.testing.assert_array_equal(a.model.state.get(name).view("i").cpu().numpy(),
                                          b.model.state.get(name).view("i").cpu().numpy(), err_msg=name)


@pytest.mark.parametrize("k", [0, 2, 3])
def test_forward_switches_to_graph_replay(k):
    """model.forward with graphs on: eager, then capture on the second call with the
    same dt, replay after; a new dt runs eagerly. Same bits as eager stepping."""
    cfg, kind, _ = CASES[k]
    dt = cfg["dt"]
    eager = _model(cfg, kind, 70 + k)
    auto = _model(cfg, kind, 70 + k, graphs=True)
    for dts in (dt, dt, dt, 0.5 * dt, dt, dt):
        eager.model.forward(0.0, dts)
        auto.model.forward(0.0, dts)
        assert auto.model.mg_stats()["nite"] == eager.model.mg_stats()["nite"]
    assert auto.model.graph == (dt, 1)
    torch.cuda.synchronize()
    _assert_same_state(auto, eager)


@pytest.mark.parametrize("k", range(len(CASES)))
def test_graph_replay_equals_eager(k):
    cfg, kind, per_graph = CASES[k]
    dt = cfg["dt"]
    eager = _model(cfg, kind, 90 + k)
    graph = _model(cfg, kind, 90 + k)
    if cfg.get("timestepping") == "LFAM3":   # the first LFAM3 step is Euler forward, eager in both
        eager.model.forward(0.0, dt)
        graph.model.forward(0.0, dt)
    graph.model.capture_graph(dt, per_graph)
    nite_e, nite_g = [], []
    for r in range(2):
        for _ in range(per_graph):
            eager.model.forward(0.0, dt)
            nite_e.append(eager.model.mg_stats()["nite"])
        graph.model.replay()
        torch.cuda.synchronize()
        nite_g.append(graph.model.mg_stats()["nite"])
    assert nite_g == nite_e[per_graph - 1::per_graph]
    assert graph.model.mg_stats()["vcycles"] == eager.model.mg_stats()["vcycles"]
    _assert_same_state(graph, eager)
