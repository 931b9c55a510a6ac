"""GPU parity of the linear tracer schemes (tracer_scheme = linear, orderA = 1..5) and
of the advection model (core/model_advection.py) against the oracle: time steps (eager
and graph replay), live diffusion of b, make_u_divergentfree, and the mixed path."""
import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def _pair(cfg, kind=None, seed=0):
    import torch
    from nyles_gb300.nyles import Nyles
    p = helpers.make_params(**cfg)
    nyl = Nyles(p)
    o = helpers.oracle_for(nyl)
    if kind is not None:
        helpers.load_state(nyl, o, helpers.seeded_state(nyl, kind, seed))
    return nyl, o, torch


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_les_linear_tracer_scheme_matches_oracle(order):
    cfg = dict(geometry="perio_xy", n=(16, 16, 16), n_tracers=1, dt=1e-3, tracer_scheme="linear", orderA=order)
    nyl, o, _ = _pair(cfg, "noise", 90 + order)
    m = nyl.model
    m.diagnose_var(m.state)
    o.diagnose()
    t = 0.0
    names = helpers.PROG + ["t0", "p"]
    for n in range(3):
        m.forward(t, 1e-3)
        o.forward(t, 1e-3)
        t += 1e-3
        assert m.mg_stats()["nite"] == o.mg_stats()[0]
        errs = helpers.parity_errors(lambda s: m.state.get(s).view("i").cpu().numpy(), o.field, names)
        for s in names:
            assert errs[s] < 1e-12 * (n + 1), (order, n, s, errs[s])


def _advection_state(nyl, o, torch, seed):
    """b: a smooth bump plus noise; U: a periodic swirl plus a vertical wave, zero
    through closed walls, its halo the periodic image (the advection model never fills
    U); u = U * dx**2. Written to the GPU model and, when given, to the oracle."""
    rng = np.random.default_rng(seed)
    g = nyl.grid
    st = nyl.model.state
    xb, yb, zb = g.x_b.view("i").numpy(), g.y_b.view("i").numpy(), g.z_b.view("i").numpy()
    b = np.exp(-((xb - 0.4) ** 2 + (yb - 0.5) ** 2 + (zb - 0.5) ** 2) / 0.02) + 1e-3 * rng.standard_normal(xb.shape)
    tp = 2.0 * np.pi
    U = {"i": 0.5 + 0.3 * np.sin(tp * yb), "j": 0.3 * np.cos(tp * xb), "k": 0.2 * np.sin(tp * xb)}
    geo = nyl.param["geometry"]
    nh = 3
    for c in "ijk":
        for axis, per in ((2, "x" in geo), (1, "y" in geo), (0, "z" in geo)):
            if per:                                # halo = periodic image of the interior
                a = np.moveaxis(U[c], axis, 0)
                n = a.shape[0] - 2 * nh
                a[:nh] = a[n:n + nh]
                a[n + nh:] = a[nh:2 * nh]
    if "x" not in geo:
        U["i"][:, :, -1] = 0.0
    if "y" not in geo:
        U["j"][:, -1, :] = 0.0
    if "z" not in geo:
        U["k"][-1, :, :] = 0.0
    fields = {"b": b}
    for c, d2 in zip("ijk", (g.dx ** 2, g.dy ** 2, g.dz ** 2)):
        fields["U_" + c] = U[c]
        fields["u_" + c] = U[c] * d2
    for k, v in fields.items():
        st.get(k).view("i")[...] = torch.from_numpy(v)
        if o is not None:
            o.field(k)[...] = v


ADV_CASES = [
    dict(geometry="closed", n=(16, 16, 16), timestepping="RK3_SSP"),
    dict(geometry="perio_xy", n=(16, 16, 16), timestepping="LFAM3", diff_coef={"b": 2e-3}),
    dict(geometry="perio_xyz", n=(16, 8, 16), timestepping="EF", diff_coef={"b": 1e-3}),
    dict(geometry="closed", n=(16, 16, 16), timestepping="RK3_SSP", tracer_scheme="linear", orderA=3,
         diff_coef={"b": 1e-3}),
]


@pytest.mark.parametrize("k", range(len(ADV_CASES)))
def test_advection_model_matches_oracle(k):
    cfg = dict(ADV_CASES[k], modelname="advection", dt=2e-3)
    nyl, o, torch = _pair(cfg)
    _advection_state(nyl, o, torch, 30 + k)
    m = nyl.model
    m.diagnose_var(m.state)
    o.diagnose()
    t = 0.0
    for n in range(6):                           # steps 2.. are graph replays
        m.forward(t, 2e-3)
        o.forward(t, 2e-3)
        t += 2e-3
    for s in ("b", "u_i", "u_j", "u_k", "U_i"):
        a = m.state.get(s).view("i").cpu().numpy()
        assert helpers.relerr(a, o.field(s)) < 1e-12 * 6, (k, s)
    np.testing.assert_array_equal(m.state.get("U_i").view("i").cpu().numpy(), o.field("U_i"))


def test_make_u_divergentfree_matches_oracle():
    cfg = dict(geometry="perio_xy", n=(16, 16, 16), modelname="advection", dt=1e-3, mg_tol=1e-12, mg_maxite=40)
    nyl, o, torch = _pair(cfg, "noise", 44)
    nyl.model.make_u_divergentfree()
    o.project()
    assert nyl.model.mg_stats()["nite"] == o.mg_stats()[0]
    names = ["u_i", "u_j", "u_k", "U_i", "U_j", "U_k", "p", "div"]
    errs = helpers.parity_errors(lambda s: nyl.model.state.get(s).view("i").cpu().numpy(), o.field, names)
    for s in names[:-1]:
        assert errs[s] < 1e-12, (s, errs[s])
    scale = np.abs(o.field("U_i")).max()
    assert helpers.relerr(nyl.model.state.div.view("i").cpu().numpy(), o.field("div"), scale) < 1e-12
    assert np.abs(o.field("div")).max() < 1e-4 * scale


def test_advection_mixed_close_to_fp64():
    import torch
    from nyles_gb300.nyles import Nyles
    runs = {}
    for prec in ("fp64", "mixed"):
        p = helpers.make_params(geometry="perio_xyz", n=(16, 16, 16), modelname="advection", dt=2e-3,
                                diff_coef={"b": 1e-3}, precision=prec)
        nyl = Nyles(p)
        _advection_state(nyl, None, torch, 7)
        m = nyl.model
        m.diagnose_var(m.state)
        for n in range(20):
            m.forward(n * 2e-3, 2e-3)
        runs[prec] = m.state.b.view("i").double().cpu().numpy()
    assert helpers.relerr(runs["mixed"], runs["fp64"]) < 1e-5


def test_advection_run_conserves_b():
    """Nyles.run on the advection model with the CFL time step: b's interior sum is
    conserved in a periodic box."""
    import torch
    from nyles_gb300.nyles import Nyles
    p = helpers.make_params(geometry="perio_xyz", n=(16, 16, 16), modelname="advection", auto_dt=True, cfl=0.5,
                            dt_max=0.05)
    p.time["tend"] = 0.2
    nyl = Nyles(p)
    _advection_state(nyl, None, torch, 9)
    nh = 3
    inner = (slice(nh, -nh),) * 3
    nyl.model.diagnose_var(nyl.model.state)
    s0 = float(nyl.model.state.b.view("i")[inner].sum())
    t, n, blowup = nyl.run(verbose=False)
    assert not blowup and t >= 0.2 and n > 1
    assert abs(float(nyl.model.state.b.view("i")[inner].sum()) - s0) < 1e-10 * abs(s0)
