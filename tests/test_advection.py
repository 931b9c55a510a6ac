"""The linear tracer schemes (core/fortran_upwind.f90:32-61 with
core/interpolate_tracer.f90) and the advection model (core/model_advection.py) in the
oracle, on the CPU. The reference never runs the linear branch (`linear = .false.`), so
there is no reference output to pin it against: the oracle is checked against an
independent numpy restatement (same operation order, bit for bit), against the
convergence order of each interpolation, and for conservation of the flux form."""
import numpy as np
import pytest

import oracle

F = np.float32


def _coefs():
    d = lambda a, b: float(F(a) / F(b))   # REAL(4) literal quotient widened to double
    return dict(c1=-d(1, 6), c2=d(5, 6), c3=d(2, 6), e1=-d(1, 12), e2=d(7, 12),
                b1=d(2, 60), b2=-d(13, 60), b3=d(47, 60), b4=d(27, 60), b5=-d(3, 60))


def upwind_linear_numpy(q, u, order):
    """dtrac of one line, restated from the Fortran loops with 1-based indices."""
    n = len(q)
    k = _coefs()
    Q = lambda i: q[i - 1]
    qp = np.zeros(n + 1)
    qm = np.zeros(n + 2)

    def cst(i):
        qp[i] = k["c1"] * Q(i - 1) + k["c2"] * Q(i) + k["c3"] * Q(i + 1)
        qm[i] = k["c3"] * Q(i - 1) + k["c2"] * Q(i) + k["c1"] * Q(i + 1)

    if order == 5:
        qp[1] = qm[1] = Q(1)
        cst(2)
        for i in range(3, n - 1):
            qp[i] = k["b1"] * Q(i - 2) + k["b2"] * Q(i - 1) + k["b3"] * Q(i) + k["b4"] * Q(i + 1) + k["b5"] * Q(i + 2)
            qm[i] = k["b5"] * Q(i - 2) + k["b4"] * Q(i - 1) + k["b3"] * Q(i) + k["b2"] * Q(i + 1) + k["b1"] * Q(i + 2)
        cst(n - 1)
        qp[n] = qm[n] = Q(n)
    elif order == 3:
        qp[1] = qm[1] = Q(1)
        for i in range(2, n):
            cst(i)
        qp[n] = qm[n] = Q(n)
    elif order == 1:
        for i in range(1, n + 1):
            qp[i] = qm[i] = Q(i)
    elif order == 2:
        for i in range(1, n):
            qp[i] = 0.5 * (Q(i) + Q(i + 1))
    elif order == 4:
        qp[1] = k["e2"] * (Q(1) + Q(2)) + k["e1"] * Q(3)
        for i in range(2, n - 1):
            qp[i] = k["e2"] * (Q(i) + Q(i + 1)) + k["e1"] * (Q(i - 1) + Q(i + 2))
        qp[n - 1] = k["e2"] * (Q(n - 1) + Q(n)) + k["e1"] * Q(n - 2)
    d = np.zeros(n)
    fxm = 0.0
    for i in range(1, n):
        ui = u[i - 1]
        if order % 2 == 0:
            fx = ui * qp[i]
        else:
            uu = abs(ui)
            fx = (0.5 * (ui + uu)) * qp[i] + (0.5 * (ui - uu)) * qm[i + 1]
        d[i - 1] = d[i - 1] + fxm - fx
        fxm = fx
    d[n - 1] = d[n - 1] + fxm - 0.0
    return d


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_linear_upwind_matches_numpy_restatement(order):
    rng = np.random.default_rng(order)
    l, m, n = 3, 4, 17
    q = rng.standard_normal((l, m, n))
    u = rng.standard_normal((l, m, n))
    d = np.zeros((l, m, n))
    oracle.upwind_linear(q, u, d, order)
    for a in range(l):
        for b in range(m):
            np.testing.assert_array_equal(d[a, b], upwind_linear_numpy(q[a, b], u[a, b], order))


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_linear_upwind_conserves(order):
    """No flux through either end: the tendencies of a line sum to zero."""
    rng = np.random.default_rng(10 + order)
    q = rng.standard_normal((2, 2, 24))
    u = rng.standard_normal((2, 2, 24))
    d = np.zeros_like(q)
    oracle.upwind_linear(q, u, d, order)
    assert np.abs(d.sum(axis=2)).max() < 1e-13


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
def test_linear_interpolation_order(order):
    """With u = 1 the face fluxes are the interpolations qp: against the exact face
    values of cell averages of sin, away from the low-order boundary closures."""
    errs = []
    hs = (0.4, 0.2, 0.1)
    for h in hs:
        n = int(round(6.0 / h))
        xc = (np.arange(n) + 0.5) * h
        q = ((np.cos(xc - h / 2) - np.cos(xc + h / 2)) / h)[None, None, :]
        d = np.zeros_like(q)
        oracle.upwind_linear(q.copy(), np.ones_like(q), d, order)
        flux = -np.cumsum(d[0, 0])               # flux(i) = flux(i-1) - dtrac(i)
        faces = np.arange(1, n + 1) * h           # right face of each cell
        inner = slice(n // 4, 3 * n // 4)
        errs.append(np.abs(flux[inner] - np.sin(faces[inner])).max())
    rates = np.log2(np.array(errs[:-1]) / np.array(errs[1:]))
    assert rates.min() > order - 0.5, (order, errs, rates)


def _advection_desc(geometry, n, timestepping="RK3_SSP", **kw):
    nx, ny, nz = n
    L = (1.0, 1.0, 1.0)
    dx, dy, dz = L[0] / nx, L[1] / ny, L[2] / nz
    return dict(nx=nx, ny=ny, nz=nz, nh=3, geometry=geometry, n_tracers=0, modelname="advection",
                timestepping=timestepping, dx=dx, dy=dy, dz=dz, idx2=1 / dx ** 2, idy2=1 / dy ** 2,
                idz2=1 / dz ** 2, **kw)


def test_advection_model_moves_b_only():
    """Advection.rhs: the tendency of b is the flux divergence by the stored U, the
    velocity tendencies are never written; diagnose_var fills b's halo only; a uniform
    U through a periodic box translates b (sum conserved, u unchanged)."""
    o = oracle.OracleModel(_advection_desc("perio_xyz", (16, 8, 8)))
    shape = o.shape
    rng = np.random.default_rng(2)
    b = rng.standard_normal(shape)
    o.field("b")[...] = b
    o.field("U_i")[...] = 0.5
    o.field("u_i")[...] = 0.5 / o.desc["idx2"]
    for q in range(4):
        o.register(0, q)[...] = 0.0
    o.register(0, 1)[...] = 7.0                  # a velocity register keeps what it holds
    o.rhs(0, last=True)
    ref = np.zeros(shape)
    oracle.upwind(np.ascontiguousarray(b), np.full(shape, 0.5), ref)
    np.testing.assert_array_equal(o.register(0, 0), ref)
    assert (o.register(0, 1) == 7.0).all() and (o.register(0, 2) == 0.0).all()
    o.register(0, 1)[...] = 0.0
    o.diagnose()                                 # fills the halo of b (Nyles.run does this first)
    nh = 3
    interior = (slice(nh, -nh),) * 3
    s0 = o.field("b")[interior].sum()
    u0 = o.field("u_i").copy()
    for k in range(5):
        o.forward(k * 0.01, 0.01)
    assert abs(o.field("b")[interior].sum() - s0) < 1e-11
    np.testing.assert_array_equal(o.field("u_i"), u0)
    h = o.field("b")
    np.testing.assert_array_equal(h[:, :, :nh], h[:, :, -2 * nh:-nh])    # halo of b filled


def test_advection_diffusion_is_live():
    """Advection.rhs passes `last`, so diff_coef['b'] diffuses b on the last stage."""
    base = _advection_desc("closed", (8, 8, 8), timestepping="EF")
    a = oracle.OracleModel(base)
    b = oracle.OracleModel(dict(base, tracer_diffusion={"b": 1e-2}))
    rng = np.random.default_rng(3)
    f = rng.standard_normal(a.shape)
    for m in (a, b):
        m.field("b")[...] = f
    a.rhs(0, last=True)
    b.rhs(0, last=False)
    np.testing.assert_array_equal(a.register(0, 0), b.register(0, 0))
    b.rhs(0, last=True)
    assert np.abs(b.register(0, 0) - a.register(0, 0)).max() > 1e-3


def test_make_u_divergentfree():
    """The projection leaves U divergence-free (to the multigrid tolerance), with
    U = u/dx**2 and the halo of div filled. Cubic cells: the reference's p = x*dx**2
    (core/mgfordriver.py:78) is exact only then."""
    o = oracle.OracleModel(_advection_desc("perio_xy", (16, 16, 16)))
    o.mg_params(1e-20, 40)
    rng = np.random.default_rng(5)
    for c in ("u_i", "u_j", "u_k"):
        o.field(c)[...] = rng.standard_normal(o.shape) * 1e-2
    o.field("u_k")[-1] = 0.0                     # closed top
    o.project()
    div = o.field("div")
    assert np.abs(div).max() < 1e-8 * np.abs(o.field("U_i")).max()
    np.testing.assert_array_equal(o.field("U_i"), o.field("u_i") * o.desc["idx2"])
