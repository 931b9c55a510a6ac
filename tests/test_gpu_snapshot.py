"""Checkpoint / resume of a run on the device: a model restored from a host snapshot
continues bit for bit like the uninterrupted run (graph replay included)."""
import numpy as np
import pytest

import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

CASES = [
    (dict(geometry="perio_xy", n=(16, 16, 32), L=(1.0, 1.0, 2.0), n_tracers=1, dt=1e-3), "noise"),
    (dict(geometry="perio_xyz", n=(16, 16, 16), L=(6.283185307179586,) * 3, modelname="Euler3d",
          timestepping="LFAM3", dt=5e-3), "tgv"),
    (dict(geometry="closed", n=(32, 16, 16), L=(2.0, 1.0, 1.0), dt=2e-3, precision="mixed"), "lock"),
]


def _model(cfg, kind):
    from nyles_gb300.nyles import Nyles
    nyl = Nyles(helpers.make_params(**cfg))
    for k, v in helpers.seeded_state(nyl, kind, 5).items():
        nyl.model.state.get(k).view("i")[...] = torch.from_numpy(v)
    nyl.model.diagnose_var(nyl.model.state)
    return nyl


@pytest.mark.parametrize("k", range(len(CASES)))
def test_restored_run_continues_identically(k):
    cfg, kind = CASES[k]
    dt = cfg["dt"]
    a = _model(cfg, kind)
    for _ in range(3):
        a.model.forward(0.0, dt)
    snap = a.model.snapshot()
    for _ in range(4):
        a.model.forward(0.0, dt)
    b = _model(cfg, kind)                 # a fresh model from the same parameters
    b.model.restore(snap)
    for _ in range(4):
        b.model.forward(0.0, dt)
    torch.cuda.synchronize()
    np.testing.assert_array_equal(a.model.state.storage.cpu().numpy(), b.model.state.storage.cpu().numpy())
    assert a.model.mg_stats()["nite"] == b.model.mg_stats()["nite"]


def test_snapshot_of_another_model_is_refused():
    a = _model(*CASES[0])
    b = _model(*CASES[2])
    with pytest.raises(ValueError):
        b.model.restore(a.model.snapshot())
