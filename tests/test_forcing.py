"""User forcing hook (core/model_les.py:143-144, `forcing.add(state, dstate, t)` after
every right-hand side): stage times and registers on the CPU oracle, and the GPU model
with a device-side forcing against the oracle with the same forcing in numpy."""
import numpy as np
import pytest

import helpers
import oracle


def _oracle(scheme):
    return oracle.OracleModel(dict(nx=16, ny=8, nz=8, geometry="closed", timestepping=scheme,
                                   dx=1 / 16, dy=1 / 8, dz=1 / 8, idx2=256.0, idy2=64.0, idz2=64.0))


@pytest.mark.parametrize("scheme,expect", [
    ("RK3_SSP", [(0, 1.0), (1, 1.5), (2, 1.25)] * 2),
    ("EF", [(0, 1.0)] * 2),
    ("LFAM3", [(0, 1.0), (0, 1.5), (0, 1.75)]),   # first step Euler; then predictor, corrector
])
def test_forcing_called_with_stage_registers_and_times(scheme, expect):
    o = _oracle(scheme)
    o.diagnose()
    calls = []
    o.set_forcing(lambda reg, t: calls.append((reg, t)))
    o.forward(1.0, 0.5)
    o.forward(1.5 if scheme == "LFAM3" else 1.0, 0.5)
    assert calls == expect


class TorchForcing:
    """Heat source Q and relaxation of b towards b0 with rate k (the shape of the
    reference's nudging example): db += Q - k*(b - b0)."""

    def __init__(self, Q, b0, k):
        import torch
        self.Q = torch.as_tensor(Q, device="cuda")
        self.b0 = torch.as_tensor(b0, device="cuda")
        self.k = k
        self.times = []

    def add(self, state, dstate, t):
        self.times.append(t)
        db = dstate.b.view("i")
        b = state.b.view("i")
        db += self.Q - self.k * (b - self.b0)


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", ["RK3_SSP", "LFAM3", "EF"])
def test_gpu_forcing_matches_oracle(scheme):
    torch = pytest.importorskip("torch")
    from nyles_gb300.nyles import Nyles
    cfg = dict(geometry="closed", n=(32, 16, 16), L=(2.0, 1.0, 1.0), dt=2e-3, timestepping=scheme, forced=True)
    nyl = Nyles(helpers.make_params(**cfg))
    o = helpers.oracle_for(nyl)
    helpers.load_state(nyl, o, helpers.seeded_state(nyl, "lock", 21))
    shape = o.field("b").shape
    rng = np.random.Generator(np.random.PCG64(3))
    Q = 1e-2 * rng.standard_normal(shape)
    b0 = o.field("b").copy()
    k = 0.3
    nyl.model.forcing = TorchForcing(Q, b0, k)

    def oracle_forcing(reg, t):
        db = o.register(reg, 0)
        b = o.field("b")
        db += Q - k * (b - b0)

    o.set_forcing(oracle_forcing)
    nyl.model.diagnose_var(nyl.model.state)
    o.diagnose()
    t = 0.0
    for _ in range(3):
        nyl.model.forward(t, cfg["dt"])
        o.forward(t, cfg["dt"])
        t += cfg["dt"]
        assert nyl.model.mg_stats()["nite"] == o.mg_stats()[0]
    torch.cuda.synchronize()
    assert nyl.model.graph is None                 # forced steps run eagerly
    names = helpers.PROG + ["p"]
    errs = helpers.parity_errors(lambda s: nyl.model.state.get(s).view("i").cpu().numpy(), o.field, names)
    for s in names:
        assert errs[s] < 1e-12, (s, errs[s])


@pytest.mark.gpu
def test_forced_model_without_forcing_raises():
    pytest.importorskip("torch")
    from nyles_gb300.nyles import Nyles
    nyl = Nyles(helpers.make_params(forced=True))
    with pytest.raises(RuntimeError):
        nyl.model.forward(0.0, 1e-3)
