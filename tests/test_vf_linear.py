"""The oracle's linear vortex-force branch against a plain-Python restatement.

core/fortran_vortex_force.f90 has a linear branch (:43-55 direc, :121-133 flip) with
the interpolation of core/interpolate.f90:3-112, which the reference never runs
(`linear = .false.` at :28 and :106; orderVF is ignored). It is selectable here
(gpu parameter vf_scheme = "linear", NylesDesc.vf_order). With no reference output for
a branch that never runs, its parity is unpinned: the oracle's C++ is checked against
this second restatement, written statement by statement from the Fortran in its own
1-based indexing, bit for bit, and against properties (a constant vorticity carried
by a constant velocity).
"""
import numpy as np
import pytest

import oracle


def _f32(a, b):
    """a REAL(4) literal quotient a./b. widened to double"""
    return float(np.float32(a) / np.float32(b))


C1, C2, C3 = _f32(-1, 6), _f32(5, 6), _f32(2, 6)
E1, E2 = _f32(-1, 12), _f32(7, 12)
B1, B2, B3, B4, B5 = _f32(2, 60), _f32(-13, 60), _f32(47, 60), _f32(27, 60), _f32(-3, 60)


def interpolate(vU, order, n):
    """core/interpolate.f90:3-112; vU, qm indexed 1..n, qp 0..n-1 (dicts)"""
    qp, qm = {}, {}
    if order == 5:
        qp[0] = 0.0
        qp[1] = vU[1]; qm[1] = vU[1]
        i = 2
        qp[i] = C1 * vU[i - 1] + C2 * vU[i] + C3 * vU[i + 1]
        qm[i] = C3 * vU[i - 1] + C2 * vU[i] + C1 * vU[i + 1]
        for i in range(3, n - 2):
            qp[i] = B1 * vU[i - 2] + B2 * vU[i - 1] + B3 * vU[i] + B4 * vU[i + 1] + B5 * vU[i + 2]
            qm[i] = B5 * vU[i - 2] + B4 * vU[i - 1] + B3 * vU[i] + B2 * vU[i + 1] + B1 * vU[i + 2]
        i = n - 2
        qp[i] = C1 * vU[i - 1] + C2 * vU[i] + C3 * vU[i + 1]
        qm[i] = C3 * vU[i - 1] + C2 * vU[i] + C1 * vU[i + 1]
        i = n - 1
        qp[i] = vU[i]; qm[i] = vU[i]
        qm[n] = vU[n]
    elif order == 3:
        qp[0] = 0.0
        qp[1] = vU[1]; qm[1] = vU[1]
        for i in range(2, n - 1):
            qp[i] = C1 * vU[i - 1] + C2 * vU[i] + C3 * vU[i + 1]
            qm[i] = C3 * vU[i - 1] + C2 * vU[i] + C1 * vU[i + 1]
        i = n - 1
        qp[i] = vU[i]; qm[i] = vU[i]
        qm[n] = vU[n]
    elif order == 1:
        qp[0] = 0.0
        for i in range(1, n):
            qp[i] = vU[i]; qm[i] = vU[i]
        qm[n] = vU[n]
    elif order == 2:
        qm[1] = 0.5 * vU[1]
        for i in range(2, n + 1):
            qm[i] = 0.5 * (vU[i - 1] + vU[i])
    elif order == 4:
        qm[1] = E2 * (vU[1]) + E1 * (vU[2])
        qm[2] = E2 * (vU[1] + vU[2]) + E1 * (vU[3])
        for i in range(3, n):
            qm[i] = E2 * (vU[i - 1] + vU[i]) + E1 * (vU[i - 2] + vU[i + 1])
        qm[n] = E2 * (vU[n - 1] + vU[n]) + E1 * (vU[n - 2])
    return qp, qm


def direc(U, vort, res, order):
    """core/fortran_vortex_force.f90:41-55 on numpy arrays (m, n, l), 0-based storage"""
    m, n, l = U.shape
    for j in range(m):
        for i in range(n - 1):
            UU_0 = 0.0
            vU, up, um = {}, {}, {}
            for k in range(1, l + 1):
                UU_1 = 0.5 * (U[j, i, k - 1] + U[j, i + 1, k - 1])
                vU[k] = vort[j, i, k - 1]
                Ui = 0.5 * (UU_0 + UU_1)
                UU = abs(Ui)
                up[k] = 0.5 * (Ui + UU)
                um[k] = 0.5 * (Ui - UU)
                UU_0 = UU_1
            qp, qm = interpolate(vU, order, l)
            for k in range(1, l + 1):
                if order % 2 == 0:
                    res[j, i, k - 1] = res[j, i, k - 1] - qm[k]
                else:
                    res[j, i, k - 1] = res[j, i, k - 1] - qp[k - 1] * up[k] - qm[k] * um[k]


def flip(U, vort, res, order):
    """core/fortran_vortex_force.f90:119-133"""
    m, n, l = U.shape
    for j in range(m):
        for k in range(l - 1):
            UU_0 = 0.0
            vU, up, um = {}, {}, {}
            for i in range(1, n + 1):
                UU_1 = 0.5 * (U[j, i - 1, k] + U[j, i - 1, k + 1])
                vU[i] = vort[j, i - 1, k]
                Ui = 0.5 * (UU_0 + UU_1)
                UU = abs(Ui)
                up[i] = 0.5 * (Ui + UU)
                um[i] = 0.5 * (Ui - UU)
                UU_0 = UU_1
            qp, qm = interpolate(vU, order, n)
            for i in range(1, n + 1):
                if order % 2 == 0:
                    res[j, i - 1, k] = res[j, i - 1, k] + qm[i]
                else:
                    res[j, i - 1, k] = res[j, i - 1, k] + qp[i - 1] * up[i] + qm[i] * um[i]


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("shape", [(3, 7, 9), (2, 6, 5), (4, 11, 6)])
def test_oracle_linear_vortex_force_matches_restatement(order, shape):
    rng = np.random.Generator(np.random.PCG64(100 * order + shape[1]))
    U = rng.standard_normal(shape)
    vort = rng.standard_normal(shape) * np.exp(rng.uniform(-3, 1, size=shape))
    res0 = rng.standard_normal(shape)
    for fn, ref_fn in ((oracle.vortex_force_direc_order, direc), (oracle.vortex_force_flip_order, flip)):
        got, ref = res0.copy(), res0.copy()
        fn(U, vort, got, order)
        ref_fn(U, vort, ref, order)
        assert np.array_equal(got, ref), (fn.__name__, order)


def test_order_zero_is_the_weno_branch():
    rng = np.random.Generator(np.random.PCG64(5))
    shape = (3, 8, 10)
    U, vort = rng.standard_normal(shape), rng.standard_normal(shape)
    a, b = np.zeros(shape), np.zeros(shape)
    oracle.vortex_force_direc_order(U, vort, a, 0)
    oracle.vortex_force_direc(U, vort, b)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("order", [1, 3, 5])
def test_constant_vorticity_carried_by_constant_velocity(order):
    """Odd orders reproduce a constant (up to the REAL(4) rounding of their
    coefficients, whose sums differ from 1 by ~1e-8): past the first point, where
    qp(0) = 0, the term is -u w0 whatever the order."""
    shape = (2, 5, 12)
    u0, w0 = 0.75, -1.5
    U = np.full(shape, u0)
    vort = np.full(shape, w0)
    res = np.zeros(shape)
    oracle.vortex_force_direc_order(U, vort, res, order)
    assert np.allclose(res[:, :-1, 1:], -u0 * w0, rtol=1e-7, atol=0)
    assert np.all(res[:, :-1, 0] == 0.0)         # qp(0) = 0 and um = 0 for u > 0
    assert np.all(res[:, -1, :] == 0.0)          # the last face of the other direction is skipped
