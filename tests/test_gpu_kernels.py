"""GPU kernels against the CPU oracle, through the C ABI (libnyles_gb300.so).

FP64 tolerances: the CUDA kernels may contract multiply-adds inside the WENO
reconstruction, so results differ from the oracle by a few units in the last place;
the bound used here is 1e-13 relative to the field's max-norm (well inside the
1e-12-per-step requirement).
"""
import ctypes

import numpy as np
import pytest

import helpers
import oracle

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL64 = 1e-13


def _lib():
    from nyles_gb300 import _native
    return _native


@pytest.mark.parametrize("n", [5, 6, 7, 8, 13, 40])
def test_flux1d_f64_matches_oracle(n):
    nat = _lib()
    rng = np.random.Generator(np.random.PCG64(n))
    nlines = 64
    u = rng.standard_normal((nlines, n))
    u[:, ::3] = np.abs(u[:, ::3])
    q = rng.standard_normal((nlines, n)) * np.exp(rng.uniform(-8, 2, size=(nlines, 1)))
    q[::7] = 1.25    # constant lines: tau5 = 0 path
    # tiny lines: tau5 below the normal float range (REAL(4) rounding to float subnormals)
    q[3::7] *= np.exp(rng.uniform(-60, -40, size=(len(q[3::7]), 1)))
    ud, qd = torch.from_numpy(u).cuda(), torch.from_numpy(q).cuda()
    fd = torch.zeros_like(ud)
    nat.check(nat.lib().nyles_flux1d_f64(ctypes.c_void_p(ud.data_ptr()), ctypes.c_void_p(qd.data_ptr()),
                                          ctypes.c_void_p(fd.data_ptr()), nlines, n, nat.stream_ptr()))
    torch.cuda.synchronize()
    got = fd.cpu().numpy()
    ref = np.stack([oracle.flux1d(u[k], q[k]) for k in range(nlines)])
    scale = np.max(np.abs(ref), axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(got - ref) / scale) < TOL64


def test_flux1d_f32_close_to_oracle():
    nat = _lib()
    rng = np.random.Generator(np.random.PCG64(7))
    nlines, n = 32, 24
    u = rng.standard_normal((nlines, n)).astype(np.float32)
    q = rng.standard_normal((nlines, n)).astype(np.float32)
    ud, qd = torch.from_numpy(u).cuda(), torch.from_numpy(q).cuda()
    fd = torch.zeros_like(ud)
    nat.check(nat.lib().nyles_flux1d_f32(ctypes.c_void_p(ud.data_ptr()), ctypes.c_void_p(qd.data_ptr()),
                                          ctypes.c_void_p(fd.data_ptr()), nlines, n, nat.stream_ptr()))
    torch.cuda.synchronize()
    ref = np.stack([oracle.flux1d(u[k].astype(np.float64), q[k].astype(np.float64)) for k in range(nlines)])
    assert np.max(np.abs(fd.cpu().numpy() - ref)) / np.max(np.abs(ref)) < 1e-5


def test_flux1d_rejects_short_lines():
    nat = _lib()
    rc = nat.lib().nyles_flux1d_f64(None, None, None, 1, 4, None)
    assert rc == nat.NYLES_BAD_ARG


CONFIGS = [
    dict(geometry="closed", n=(16, 8, 12)),
    dict(geometry="perio_xy", n=(8, 16, 8), n_tracers=2),
    dict(geometry="perio_xyz", n=(8, 8, 8)),
    dict(geometry="perio_x", n=(12, 8, 8)),
    dict(geometry="closed", n=(8, 8, 8), modelname="Euler3d"),
    dict(geometry="perio_xy", n=(8, 8, 8), modelname="linear", n_tracers=1),
    dict(geometry="closed", n=(8, 8, 8), rotating=True, coriolis=3.0, diff_coef={"u": 2e-3}),
]


def _setup(cfg, seed):
    from nyles_gb300.nyles import Nyles
    p = helpers.make_params(**cfg)
    nyl = Nyles(p)
    o = helpers.oracle_for(nyl)
    fields = helpers.seeded_state(nyl, "noise", seed)
    helpers.load_state(nyl, o, fields)
    return nyl, o


def _fill_random_diagnostics(nyl, o, seed):
    """Random U, vor, ke (the inputs of the right-hand side), identical on both sides."""
    rng = np.random.Generator(np.random.PCG64(seed))
    shape = tuple(nyl.model.state.b.view("i").shape)
    for name in ("U_i", "U_j", "U_k", "vor_i", "vor_j", "vor_k", "ke"):
        a = rng.standard_normal(shape)
        if name.startswith("vor"):
            a *= np.exp(rng.uniform(-6, 0, size=shape))
        nyl.model.state.get(name).view("i")[...] = torch.from_numpy(a)
        o.field(name)[...] = a


@pytest.mark.parametrize("k", range(len(CONFIGS)))
def test_vortex_force_f64_matches_oracle(k):
    nat = _lib()
    nyl, o = _setup(CONFIGS[k], 10 + k)
    _fill_random_diagnostics(nyl, o, 20 + k)
    m = nyl.model
    ds = m.timescheme.registers[0]
    ds.storage.zero_()
    fields = nat.ptr_array([s.data_ptr() for s in m.state.scalars()])
    dsp = nat.ptr_array([s.data_ptr() for s in ds.scalars()])
    nat.check(nat.lib().nyles_vortex_force_f64(ctypes.byref(m.desc), fields, dsp, nat.stream_ptr()))
    torch.cuda.synchronize()
    o.vortex_force(0)
    for q, name in enumerate(["u_i", "u_j", "u_k"]):
        got = ds.get(name).view("i").cpu().numpy()
        ref = o.register(0, 1 + q)
        assert helpers.relerr(got, ref) < TOL64, name


@pytest.mark.parametrize("order", [1, 2, 3, 4, 5])
@pytest.mark.parametrize("k", [0, 1, 2])
def test_vortex_force_linear_matches_oracle(k, order):
    """The linear branch of core/fortran_vortex_force.f90 (vf_order = orderVF), FP64 at
    the kernel bar and FP32 within 1e-5 of the FP64 oracle."""
    nat = _lib()
    for prec in ("fp64", "mixed"):
        cfg = dict(CONFIGS[k], vf_scheme="linear", orderVF=order, precision=prec)
        nyl, o = _setup(cfg, 50 + k)
        _fill_random_diagnostics(nyl, o, 60 + k)
        m = nyl.model
        assert m.desc.vf_order == order
        ds = m.timescheme.registers[0]
        ds.storage.zero_()
        fields = nat.ptr_array([s.data_ptr() for s in m.state.scalars()])
        dsp = nat.ptr_array([s.data_ptr() for s in ds.scalars()])
        fn = nat.lib().nyles_vortex_force_f64 if prec == "fp64" else nat.lib().nyles_vortex_force_f32
        nat.check(fn(ctypes.byref(m.desc), fields, dsp, nat.stream_ptr()))
        torch.cuda.synchronize()
        o.vortex_force(0)
        for q, name in enumerate(["u_i", "u_j", "u_k"]):
            got = ds.get(name).view("i").double().cpu().numpy()
            ref = o.register(0, 1 + q)
            assert helpers.relerr(got, ref) < (TOL64 if prec == "fp64" else 1e-5), (prec, name)


@pytest.mark.parametrize("order", [2, 5])
@pytest.mark.parametrize("k", [0, 1])
def test_rhs_with_linear_vortex_force_matches_oracle(k, order):
    nyl, o = _setup(dict(CONFIGS[k], vf_scheme="linear", orderVF=order), 70 + k)
    _fill_random_diagnostics(nyl, o, 80 + k)
    m = nyl.model
    ds = m.timescheme.registers[1]
    ds.storage.fill_(123.0)
    m.rhs(m.state, 0.0, ds, last=True)
    torch.cuda.synchronize()
    o.rhs(1, True)
    for q, name in enumerate(["b", "u_i", "u_j", "u_k"] + ["t%d" % t for t in range(nyl.param["n_tracers"])]):
        got = ds.get(name).view("i").cpu().numpy()
        assert helpers.relerr(got, o.register(1, q)) < TOL64, name


def test_vf_order_out_of_range_is_refused():
    nat = _lib()
    nyl, o = _setup(CONFIGS[0], 1)
    d = nat.NylesDesc.from_buffer_copy(nyl.model.desc)
    d.vf_order = 6
    rc = nat.lib().nyles_vortex_force_f64(ctypes.byref(d), nat.ptr_array([0] * 14), nat.ptr_array([0] * 4), None)
    assert rc == nat.NYLES_BAD_ARG and b"vf_order" in nat.lib().nyles_last_error()


@pytest.mark.parametrize("last", [False, True])
@pytest.mark.parametrize("k", range(len(CONFIGS)))
def test_rhs_f64_matches_oracle(k, last):
    nyl, o = _setup(CONFIGS[k], 30 + k)
    _fill_random_diagnostics(nyl, o, 40 + k)
    m = nyl.model
    ds = m.timescheme.registers[1]
    ds.storage.fill_(123.0)          # overwritten entirely (reset_state)
    m.rhs(m.state, 0.0, ds, last=last)
    torch.cuda.synchronize()
    o.rhs(1, last)
    names = ["b", "u_i", "u_j", "u_k"] + ["t%d" % t for t in range(nyl.param["n_tracers"])]
    for q, name in enumerate(names):
        got = ds.get(name).view("i").cpu().numpy()
        ref = o.register(1, q)
        if np.max(np.abs(ref)) == 0:
            assert np.max(np.abs(got)) == 0, name
        else:
            assert helpers.relerr(got, ref) < TOL64, name


@pytest.mark.parametrize("k", range(len(CONFIGS)))
def test_diagnose_f64_matches_oracle(k):
    """Halo fill + divergence + multigrid + correction + vorticity + ke."""
    nyl, o = _setup(CONFIGS[k], 50 + k)
    m = nyl.model
    m.diagnose_var(m.state)
    torch.cuda.synchronize()
    o.diagnose()
    assert m.mg_stats()["nite"] == o.mg_stats()[0]
    for name in helpers.PROG + helpers.DIAG:
        got = m.state.get(name).view("i").cpu().numpy()
        ref = o.field(name)
        assert helpers.relerr(got, ref) < 1e-12, name


def test_fill_matches_oracle():
    nat = _lib()
    nyl, o = _setup(dict(geometry="perio_xyz", n=(8, 8, 8)), 3)
    m = nyl.model
    rng = np.random.Generator(np.random.PCG64(5))
    a = rng.standard_normal(tuple(m.state.ke.view("i").shape))
    m.state.ke.view("i")[...] = torch.from_numpy(a)
    o.field("ke")[...] = a
    nat.check(nat.lib().nyles_fill_f64(ctypes.byref(m.desc), ctypes.c_void_p(m.state.ke.data_ptr()), nat.stream_ptr()))
    torch.cuda.synchronize()
    o.fill("ke")
    np.testing.assert_array_equal(m.state.ke.view("i").cpu().numpy(), o.field("ke"))


_RHS_CODE = (
    "import sys, numpy as np, torch\n"
    "sys.path.insert(0, 'tests')\n"
    "import helpers\n"
    "from nyles_gb300.nyles import Nyles\n"
    "out = []\n"
    "cases = [dict(geometry='closed', n=(16, 8, 12)), dict(geometry='perio_xy', n=(48, 24, 32)),\n"
    "         dict(geometry='perio_xyz', n=(8, 8, 8)), dict(geometry='perio_x', n=(48, 8, 8)),\n"
    "         dict(geometry='closed', n=(64, 16, 16), modelname='Euler3d'),\n"
    "         dict(geometry='closed', n=(8, 8, 8), diff_coef={'u': 2e-3})]\n"
    "for prec in ('fp64', 'mixed'):\n"
    "    for k, cfg in enumerate(cases):\n"
    "        nyl = Nyles(helpers.make_params(precision=prec, **cfg))\n"
    "        m = nyl.model\n"
    "        rng = np.random.Generator(np.random.PCG64(70 + k))\n"
    "        for s in m.state.scalars():\n"
    "            a = rng.standard_normal(tuple(s.data.shape))\n"
    "            s.data.copy_(torch.from_numpy(a))\n"
    "        for last in (False, True):\n"
    "            ds = m.timescheme.registers[1]\n"
    "            ds.storage.fill_(123.0)\n"
    "            m.rhs(m.state, 0.0, ds, last=last)\n"
    "            torch.cuda.synchronize()\n"
    "            out += [ds.get(q).view('i').double().cpu().numpy() for q in ('b', 'u_i', 'u_j', 'u_k')]\n"
    "np.savez(sys.argv[1], *out)\n")


def _rhs_outputs(tmp_path, tag, **env_extra):
    """right-hand sides of seeded random states (every field drawn) on closed and
    periodic grids, FP64 and FP32, in a fresh process with the given environment"""
    import os
    import subprocess
    import sys
    root = os.path.dirname(helpers.HERE)
    env = dict(os.environ, PYTHONPATH=root, **env_extra)
    fn = str(tmp_path / ("rhs_%s.npz" % tag))
    r = subprocess.run([sys.executable, "-c", _RHS_CODE, fn], env=env, capture_output=True, text=True, cwd=root)
    assert r.returncode == 0, r.stderr[-2000:]
    with np.load(fn) as f:
        return [f["arr_%d" % i] for i in range(len(f.files))]


def test_rhs_32bit_offsets_kernel_matches_generic_kernel(tmp_path):
    """k_rhs_les (32-bit offsets, six-value loads, neighbour-shared velocity averages)
    against k_rhs_march (NYLES_GB300_GENERIC_RHS=1): the same operations in the same
    order, near array ends (closure branches) and in the interior. The compiler fuses
    multiply-adds differently in the two kernels, so values agree to rounding: 1e-5 of
    the max-norm in FP32. The FP64 right-hand side runs k_rhs_march either way (the
    FP64 cases must agree bit for bit)."""
    new = _rhs_outputs(tmp_path, "les")
    old = _rhs_outputs(tmp_path, "generic", NYLES_GB300_GENERIC_RHS="1")
    assert len(new) == len(old) == 2 * 6 * 2 * 4
    half = len(new) // 2          # FP64 cases first, then mixed
    for k, (a, b) in enumerate(zip(new, old)):
        if k < half:
            np.testing.assert_array_equal(a, b, err_msg=str(k))
        else:
            assert helpers.relerr(a, b) < 1e-5, k
