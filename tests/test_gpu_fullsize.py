"""The configurations at their full sizes on one GPU.

* Taylor-Green 128^3 (triply periodic, WENO5, RK3, dt = 5e-3, relative residual 1e-10):
  the initial projection and one step against the oracle at the FP64 bar, equal V-cycle
  counts (the oracle needs about half a minute for it).
* Rayleigh-Taylor 256^3 (the bench workload) and 256 x 256 x 512 (its specified box),
  FP64 and mixed: size-independent properties — the buoyancy integral is conserved by
  the flux-form advection to round-off, and the projection leaves a divergence at the
  multigrid tolerance (FP64) or at FP32 round-off (mixed).
* Stratified shear with a passive tracer, 512 x 256 x 256, mixed, adaptive CFL: the
  tracer integral is conserved and the CFL step follows the velocity.
"""
import numpy as np
import pytest

import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TWO_PI = 6.283185307179586


def test_taylor_green_128_step_matches_oracle():
    from nyles_gb300.nyles import Nyles
    cfg = dict(geometry="perio_xyz", n=(128, 128, 128), L=(TWO_PI,) * 3, dt=5e-3, mg_tol=1e-20, mg_maxite=40)
    nyl = Nyles(helpers.make_params(**cfg))
    o = helpers.oracle_for(nyl)
    helpers.load_state(nyl, o, helpers.seeded_state(nyl, "tgv", 2))
    nyl.model.diagnose_var(nyl.model.state)
    o.diagnose()
    assert nyl.model.mg_stats()["nite"] == o.mg_stats()[0]
    t = 0.0
    for n in range(1):
        nyl.model.forward(t, cfg["dt"])
        o.forward(t, cfg["dt"])
        t += cfg["dt"]
        assert nyl.model.mg_stats()["nite"] == o.mg_stats()[0]
        names = helpers.PROG + ["p"]
        errs = helpers.parity_errors(lambda s: nyl.model.state.get(s).view("i").cpu().numpy(), o.field, names)
        for s in names:
            assert errs[s] < 1e-12 * (n + 1), (n, s, errs[s])


def _interior(nyl, a):
    k0, k1, j0, j1, i0, i1 = nyl.grid.domainindices
    return a[k0:k1, j0:j1, i0:i1]


def _div_rms(nyl):
    """RMS over the interior of the divergence of U = u / dx^2 (float64 on the host)."""
    g = nyl.grid
    st = nyl.model.state
    U = [st.get("u_" + c).view("i").double().cpu().numpy() * f for c, f in zip("ijk", (g.idx2, g.idy2, g.idz2))]
    d = np.zeros_like(U[0])
    d[:, :, 1:] += U[0][:, :, 1:] - U[0][:, :, :-1]
    d[:, 1:, :] += U[1][:, 1:, :] - U[1][:, :-1, :]
    d[1:, :, :] += U[2][1:, :, :] - U[2][:-1, :, :]
    if "z" not in nyl.param["geometry"]:
        d[0, :, :] += U[2][0, :, :]
    return float(np.sqrt((_interior(nyl, d) ** 2).mean()))


@pytest.mark.parametrize("n", [(256, 256, 256), (256, 256, 512)])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_rayleigh_taylor_conservation_and_divergence(n, precision):
    import bench
    from nyles_gb300.nyles import Nyles
    p = bench.rt_params(n[0], precision)
    p.discretization["global_nz"] = n[2]
    p.model["Lz"] = n[2] / n[0]
    nyl = Nyles(p)
    bench.rt_init(nyl)
    m = nyl.model
    m.diagnose_var(m.state)
    b0 = _interior(nyl, m.state.b.view("i").double().cpu().numpy()).sum()
    scale = _interior(nyl, np.abs(m.state.b.view("i").double().cpu().numpy())).sum()
    for _ in range(3):
        m.forward(0.0, 1e-3)
    torch.cuda.synchronize()
    b1 = _interior(nyl, m.state.b.view("i").double().cpu().numpy()).sum()
    tol_mass = 1e-12 if precision == "fp64" else 1e-5
    assert abs(b1 - b0) <= tol_mass * scale, (b1 - b0, scale)
    # divergence left by the last projection against the velocity scale
    g = nyl.grid
    umax = max(float(m.state.get("u_" + c).view("i").abs().max()) * f
               for c, f in zip("ijk", (g.idx2, g.idy2, g.idz2)))
    div = _div_rms(nyl)
    assert div <= (1e-9 if precision == "fp64" else 1e-5) * umax, (div, umax)
    assert m.mg_stats()["not_converged"] == 0


def test_shear_tracer_512_mixed_adaptive_cfl():
    from nyles_gb300.nyles import Nyles
    cfg = dict(geometry="perio_xy", n=(512, 256, 256), L=(4.0, 2.0, 1.0), n_tracers=1, precision="mixed",
               auto_dt=True, cfl=0.8, dt_max=1.0)
    nyl = Nyles(helpers.make_params(**cfg))
    g = nyl.grid
    st = nyl.model.state
    rng = np.random.Generator(np.random.PCG64(4))
    zb = g.z_b.view("i").numpy()
    zu = g.z_vel["i"].view("i").numpy()
    U0 = 0.05 * np.sqrt(5.0)
    shape = zb.shape
    st.get("u_i").view("i")[...] = torch.from_numpy(U0 * np.tanh((zu - 0.5) / 0.05) * g.dx)
    st.get("b").view("i")[...] = torch.from_numpy(zb.copy())
    st.get("t0").view("i")[...] = torch.from_numpy(np.tanh((zb - 0.5) / 0.05))
    v = 1e-3 * rng.standard_normal(shape) * g.dy
    w = 1e-3 * rng.standard_normal(shape) * g.dz
    w[-1, :, :] = 0.0
    st.get("u_j").view("i")[...] = torch.from_numpy(v)
    st.get("u_k").view("i")[...] = torch.from_numpy(w)
    t0 = _interior(nyl, st.get("t0").view("i").double().cpu().numpy()).sum()
    t, n, blowup = nyl.run(nsteps=4, verbose=False)
    assert not blowup and n == 4
    dt = nyl.compute_dt()
    assert 0.0 < dt < 1.0                       # set by the CFL number, not dt_max
    t1 = _interior(nyl, st.get("t0").view("i").double().cpu().numpy()).sum()
    scale = _interior(nyl, np.abs(st.get("t0").view("i").double().cpu().numpy())).sum()
    assert abs(t1 - t0) <= 1e-5 * scale
