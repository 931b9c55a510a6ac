"""Known-answer checks of the oracle's kernel restatements (the reference ships no
golden vectors for its Fortran kernels; these are its __main__ demos plus analytic
properties)."""
import numpy as np
import pytest

import oracle


def test_weno5_constant_and_linear():
    # The REAL(4) literals of core/weno.f90:35-37 (1./3., 7./6., ...) do not sum to one
    # in double precision: a constant is reproduced to ~4.5e-9 only, as in the reference.
    for c in (1.0, -3.5, 1e-3):
        w = oracle.weno5(c, c, c, c, c)
        assert w != c
        assert w == pytest.approx(c, rel=1e-8)
        assert oracle.weno3(c, c, c) == c          # weno3 uses exact literals
    assert oracle.weno5(0.0, 0.0, 0.0, 0.0, 0.0) == 0.0
    # a linear profile q_i = i reconstructed at the right face of cell 0 gives 0.5
    assert oracle.weno5(-2, -1, 0, 1, 2) == pytest.approx(0.5, rel=1e-7)


def test_weno5_fifth_order_on_smooth_data():
    errs = []
    for h in (0.1, 0.05, 0.025):
        x = np.array([-2, -1, 0, 1, 2]) * h
        # cell averages of sin over [x-h/2, x+h/2]
        q = (np.cos(x - h / 2) - np.cos(x + h / 2)) / h
        errs.append(abs(oracle.weno5(*q) - np.sin(h / 2)))
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert rates.min() > 4.0   # close to 5 (tau5 rounding and eps keep it below)


def test_flux1d_closures_and_upwinding():
    n = 12
    q = np.linspace(0.0, 1.0, n) ** 2
    up = np.ones(n)
    f = oracle.flux1d(up, q)
    assert f[-1] == 0.0
    assert f[0] == q[0]                                   # first order at the left end (u > 0)
    assert f[1] == pytest.approx(oracle.weno3(q[0], q[1], q[2]))
    assert f[5] == pytest.approx(oracle.weno5(q[3], q[4], q[5], q[6], q[7]))
    fm = oracle.flux1d(-up, q)
    assert fm[n - 2] == -q[n - 1]                         # first order at the right end (u < 0)
    assert fm[5] == pytest.approx(-oracle.weno5(q[8], q[7], q[6], q[5], q[4]))


def test_kinetic_energy_constant_velocity():
    """core/kinenergy.py:28-83: with constant u0, v0, w0, max(ke) = 1/2(u0^2/dx^2+...)."""
    l, m, n = 6, 7, 8
    u0, v0, w0 = 0.3, -0.2, 0.5
    dx, dy, dz = 0.1, 0.2, 0.25
    ke = np.zeros((l, m, n))
    # view('i'): x innermost
    oracle.kin(np.full((l, m, n), u0), ke, 1 / dx ** 2)
    kt = np.ascontiguousarray(ke.transpose(2, 0, 1))          # view('j'): (x, z, y)
    oracle.kin(np.full(kt.shape, v0), kt, 1 / dy ** 2)
    ke = np.ascontiguousarray(kt.transpose(1, 2, 0))
    kk = np.ascontiguousarray(ke.transpose(1, 2, 0))          # view('k'): (y, x, z)
    oracle.kin(np.full(kk.shape, w0), kk, 1 / dz ** 2)
    ke = np.ascontiguousarray(kk.transpose(2, 0, 1))
    expect = 0.5 * (u0 ** 2 / dx ** 2 + v0 ** 2 / dy ** 2 + w0 ** 2 / dz ** 2)
    assert ke.max() == pytest.approx(expect, rel=1e-14)
    # the first cell along each direction misses that direction's contribution
    assert ke[0, 0, 0] == 0.0


def test_solid_body_rotation_vorticity():
    """core/vorticity.py:60-111: solid-body rotation has uniform vorticity 2*Omega."""
    n = 16
    dx = 1.0 / n
    Omega = 0.7
    x = (np.arange(n) + 0.5) * dx
    y = (np.arange(n) + 0.5) * dx
    # covariant velocities at faces: u = -Omega*(y-yc)*dx, v = Omega*(x-xc)*dx
    X, Y = np.meshgrid(x + dx / 2, y, indexing="xy")
    u = np.broadcast_to(-Omega * (Y - 0.5) * dx, (4, n, n)).copy()
    X, Y = np.meshgrid(x, y + dx / 2, indexing="xy")
    v = np.broadcast_to(Omega * (X - 0.5) * dx, (4, n, n)).copy()
    wk = np.zeros((4, n, n))
    oracle.vorticity(u, v, wk)
    inner = wk[:, :-1, :-1] / dx ** 2
    assert np.allclose(inner, 2 * Omega, rtol=1e-12)
    assert np.all(wk[:, :-1, -1] == 0.0)


def test_tracer_flux_form_conserves_mass_closed():
    rng = np.random.Generator(np.random.PCG64(3))
    l, m, n = 5, 6, 20
    trac = rng.standard_normal((l, m, n))
    u = rng.standard_normal((l, m, n))
    u[:, :, -1] = 0.0        # wall face
    dtrac = np.zeros_like(trac)
    oracle.upwind(trac, u, dtrac)
    assert abs(dtrac.sum()) < 1e-12 * np.abs(dtrac).sum()


@pytest.mark.parametrize("topology", [1, 5, 6])
def test_multigrid_point_sources_converge_monotonically(topology):
    """core/mgfor/tests.f90:50-57: two opposite point sources."""
    mg = oracle.OracleMG(16, 16, 16, topology)
    mg.params(tol=1e-20, maxite=1, omega=0.9)
    b = np.zeros(mg.shape())
    b[3 + 3, 3 + 3, 3 + 1] = 1.0
    b[3 + 10, 3 + 9, 3 + 4] = -1.0
    mg.set(2, b)
    res = []
    for _ in range(8):
        nite, r = mg.solve()
        res.append(r)
    assert all(res[i + 1] < res[i] for i in range(len(res) - 1))
    assert res[-1] < 1e-6 * res[0]


def test_multigrid_hierarchy_sizes():
    assert oracle.OracleMG(64, 32, 32, 1).nlevels == 5
    assert oracle.OracleMG(128, 128, 128, 6).nlevels == 7
    assert oracle.OracleMG(48, 48, 48, 1).nlevels == 5     # stops at the odd extent 3


def test_compute_dt_cases():
    """core/nyles.py:306-321: dt = cfl/|U| (or dt_max when U = 0)."""
    o = oracle.OracleModel(dict(nx=8, ny=8, nz=8, geometry="closed", dx=1.0, dy=1.0, dz=1.0,
                                idx2=1.0, idy2=1.0, idz2=1.0))
    cfl, dt_max = 0.8, 1.5
    assert o.compute_dt(True, 0.1, cfl, dt_max) == dt_max
    o.field("U_i")[...] = 1.0
    assert o.compute_dt(True, 0.1, cfl, dt_max) == pytest.approx(cfl)
    o.field("U_j")[...] = 1.0
    assert o.compute_dt(True, 0.1, cfl, dt_max) == pytest.approx(cfl / np.sqrt(2))
    o.field("U_k")[...] = 1.0
    assert o.compute_dt(True, 0.1, cfl, dt_max) == pytest.approx(cfl / np.sqrt(3))
    assert o.compute_dt(False, 0.1, cfl, dt_max) == 0.1


def test_tracer_diffusion_adds_laplacians_on_last_stage():
    """Opt-in tracer diffusion (core/tracer.py:74-76): on the last stage the tendency of
    each named tracer gains sum_d kappa*ids2[d]*(phi[i+1]-2phi[i]+phi[i-1]) with no flux
    through the array ends (core/fortran_dissipation.f90:2-35); tracers without a
    coefficient and the velocity are unchanged, and without `last` nothing changes."""
    nx, ny, nz = 8, 6, 5
    L = (2.0, 1.5, 1.0)
    dx, dy, dz = L[0] / nx, L[1] / ny, L[2] / nz
    base = dict(nx=nx, ny=ny, nz=nz, nh=3, geometry="closed", n_tracers=2, modelname="LES",
                timestepping="RK3_SSP", dx=dx, dy=dy, dz=dz, idx2=1 / dx ** 2, idy2=1 / dy ** 2, idz2=1 / dz ** 2)
    kappa = {"b": 1e-2, "t1": 3e-3}
    plain = oracle.OracleModel(base)
    diff = oracle.OracleModel(dict(base, tracer_diffusion=kappa))
    rng = np.random.default_rng(4)
    for name in ("b", "t0", "t1", "u_i", "u_j", "u_k"):
        a = rng.standard_normal(plain.shape)
        plain.field(name)[...] = a
        diff.field(name)[...] = a
    for m in (plain, diff):
        m.diagnose()
    plain.rhs(0, last=True)
    diff.rhs(0, last=False)
    for q in range(6):                           # b, u_i, u_j, u_k, t0, t1
        np.testing.assert_array_equal(diff.register(0, q), plain.register(0, q))
    diff.rhs(0, last=True)

    def lap(phi, axis, coef):
        f = np.diff(phi, axis=axis)
        pad = [(0, 0)] * 3
        pad[axis] = (1, 1)
        f = np.pad(f, pad)                       # zero flux through both array ends
        return coef * np.diff(f, axis=axis)

    for q, name in ((0, "b"), (5, "t1")):
        phi = diff.field(name)
        expect = sum(lap(phi, ax, kappa[name] * c) for ax, c in ((2, 1 / dx ** 2), (1, 1 / dy ** 2), (0, 1 / dz ** 2)))
        np.testing.assert_allclose(diff.register(0, q) - plain.register(0, q), expect, rtol=1e-9, atol=1e-12)
    for q in (1, 2, 3, 4):                       # u_i, u_j, u_k and t0 (no coefficient)
        np.testing.assert_array_equal(diff.register(0, q), plain.register(0, q))
