"""CPU oracle for the Nyles LES time step — TEST INFRASTRUCTURE ONLY.

ctypes wrapper around ``oracle/_build/libnyles_oracle.so`` (a C++ restatement of the
reference's Fortran kernels, of mgfor, and of the Python orchestration in
core/model_les.py, core/timescheme.py, core/projection.py; its loops may run on several
host threads with identical results).
Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this module, and only as the checker. The product path never does.

Parity status: partially pinned. Orchestration is pinned against the reference's
own Python modules (tests/golden/make_golden.py); the Fortran kernel restatements
are checked with the reference's known-answer demos and analytic properties,
because no Fortran compiler exists in this environment.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libnyles_oracle.so")
_lib = None

# field ids of the oracle model (state.toc order of core/variables.py:38-47)
FIELDS = {"b": 0, "p": 1, "ke": 2, "div": 3, "u_i": 4, "u_j": 5, "u_k": 6,
          "U_i": 7, "U_j": 8, "U_k": 9, "vor_i": 10, "vor_j": 11, "vor_k": 12,
          "work": 13}
SCHEMES = {"EF": 0, "LFAM3": 1, "RK3_SSP": 2}
MODELS = {"LES": 0, "Euler3d": 1, "linear": 2, "advection": 3}
# mg_enums.f90:6
MG_TOPOLOGY = {"closed": 1, "perio_x": 2, "perio_y": 3, "perio_xy": 5, "perio_xyz": 6}


def build():
    """Compile the oracle library with its Makefile (g++, -ffp-contract=off)."""
    subprocess.run(["make", "-s", "-C", _HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        src = os.path.join(_HERE, "nyles_oracle.cpp")
        if (not os.path.exists(_SO)) or os.path.getmtime(_SO) < os.path.getmtime(src):
            build()
        L = ctypes.CDLL(_SO)
        d, i, p, v = ctypes.c_double, ctypes.c_int, ctypes.c_void_p, None
        dp = ctypes.POINTER(ctypes.c_double)
        sig = {
            "orc_set_threads": (i, [i]),
            "orc_get_threads": (i, []),
            "orc_weno3": (d, [d, d, d]),
            "orc_weno5": (d, [d, d, d, d, d]),
            "orc_flux1d": (v, [p, p, p, i]),
            "orc_vortex_force_direc": (v, [p, p, p, i, i, i]),
            "orc_vortex_force_flip": (v, [p, p, p, i, i, i]),
            "orc_upwind": (v, [p, p, p, i, i, i]),
            "orc_upwind_linear": (v, [p, p, p, i, i, i, i]),
            "orc_vorticity": (v, [p, p, p, i, i, i]),
            "orc_kin": (v, [p, p, d, i, i, i]),
            "orc_gradke": (v, [p, p, i, i, i]),
            "orc_gradkeandb": (v, [p, p, p, d, i, i, i]),
            "orc_div": (v, [p, p, i, i, i, i]),
            "orc_add_laplacian": (v, [p, p, d, i, i, i]),
            "orc_mg_create": (p, [i, i, i, i]),
            "orc_mg_destroy": (v, [p]),
            "orc_mg_nlevels": (i, [p]),
            "orc_mg_shape": (v, [p, i, p]),
            "orc_mg_get": (v, [p, i, i, p]),
            "orc_mg_set": (v, [p, i, i, p]),
            "orc_mg_params": (v, [p, d, i, d]),
            "orc_mg_solve": (v, [p, p, p]),
            "orc_mg_vcycle": (v, [p]),
            "orc_mg_smooth": (v, [p, i]),
            "orc_mg_residual": (v, [p, i]),
            "orc_mg_restrict": (v, [p, i]),
            "orc_mg_prolong": (v, [p, i]),
            "orc_mg_norm": (d, [p, i, i]),
            "orc_model_create": (p, [i, i, i, i, i, i, i, i, d, d, d, d, d, d, d, d, i, i]),
            "orc_model_destroy": (v, [p]),
            "orc_model_field": (dp, [p, i]),
            "orc_model_reg": (dp, [p, i, i]),
            "orc_model_mg_params": (v, [p, d, i, d]),
            "orc_model_mg_stats": (v, [p, p, p]),
            "orc_model_mg": (p, [p]),
            "orc_model_diagnose": (v, [p]),
            "orc_model_rhs": (v, [p, i, i]),
            "orc_model_vortex_force": (v, [p, i]),
            "orc_model_forward": (v, [p, d, d]),
            "orc_model_fill": (v, [p, i]),
            "orc_model_max_U2": (d, [p]),
            "orc_model_vfwork": (d, [p, p]),
            "orc_model_set_forcing": (v, [p, p, p]),
            "orc_model_set_tracer_diffusion": (v, [p, p, i]),
            "orc_model_set_tracer_order": (v, [p, i]),
            "orc_model_set_vf_order": (v, [p, i]),
            "orc_vortex_force_direc_order": (v, [p, p, p, i, i, i, i]),
            "orc_vortex_force_flip_order": (v, [p, p, p, i, i, i, i]),
            "orc_model_project": (v, [p]),
        }
        for name, (res, args) in sig.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def set_threads(n):
    """Host threads of the oracle's parallel loops (n <= 0: all hardware threads).
    Results do not depend on it: the loops split into chunks that write disjoint
    elements, and the sums stay sequential."""
    return lib().orc_set_threads(int(n))


def threads():
    return lib().orc_get_threads()


def _ptr(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"], "oracle kernels take C-contiguous float64"
    return a.ctypes.data


# ------------------------------------------------------------------ kernels (f2py shape)
def weno3(qm, q0, qp):
    return lib().orc_weno3(qm, q0, qp)


def weno5(qmm, qm, q0, qp, qpp):
    return lib().orc_weno5(qmm, qm, q0, qp, qpp)


def flux1d(u, q):
    u = np.ascontiguousarray(u, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    out = np.zeros_like(u)
    lib().orc_flux1d(_ptr(u), _ptr(q), _ptr(out), u.size)
    return out


def vortex_force_direc(U, vort, res):
    lib().orc_vortex_force_direc(_ptr(U), _ptr(vort), _ptr(res), *res.shape)


def vortex_force_flip(U, vort, res):
    lib().orc_vortex_force_flip(_ptr(U), _ptr(vort), _ptr(res), *res.shape)


def vortex_force_direc_order(U, vort, res, order):
    """core/fortran_vortex_force.f90 vortex_force_direc with `order` honoured: 0 = the
    WENO branch (the reference's), 1..5 = its linear branch with core/interpolate.f90"""
    lib().orc_vortex_force_direc_order(_ptr(U), _ptr(vort), _ptr(res), int(order), *res.shape)


def vortex_force_flip_order(U, vort, res, order):
    lib().orc_vortex_force_flip_order(_ptr(U), _ptr(vort), _ptr(res), int(order), *res.shape)


def upwind(trac, u, dtrac):
    lib().orc_upwind(_ptr(trac), _ptr(u), _ptr(dtrac), *dtrac.shape)


def upwind_linear(trac, u, dtrac, order):
    """the linear branch of core/fortran_upwind.f90:32-61 with core/interpolate_tracer.f90"""
    lib().orc_upwind_linear(_ptr(trac), _ptr(u), _ptr(dtrac), int(order), *dtrac.shape)


def vorticity(ui, uj, wk):
    lib().orc_vorticity(_ptr(ui), _ptr(uj), _ptr(wk), *wk.shape)


def kin(u, ke, ds2):
    lib().orc_kin(_ptr(u), _ptr(ke), float(ds2), *ke.shape)


def gradke(ke, du):
    lib().orc_gradke(_ptr(ke), _ptr(du), *du.shape)


def gradkeandb(ke, b, du, dz):
    lib().orc_gradkeandb(_ptr(ke), _ptr(b), _ptr(du), float(dz), *du.shape)


def div(d, u, iflag):
    lib().orc_div(_ptr(d), _ptr(u), int(iflag), *d.shape)


def add_laplacian(phi, dphi, coef):
    lib().orc_add_laplacian(_ptr(phi), _ptr(dphi), float(coef), *dphi.shape)


# ------------------------------------------------------------------ multigrid
class OracleMG:
    """mgfor for one rank (core/mgfor/mg_setup.f90:318-437, solvers.f90:8-55)."""

    def __init__(self, nx, ny, nz, topology=1):
        self.h = lib().orc_mg_create(nx, ny, nz, topology)
        self.nlevels = lib().orc_mg_nlevels(self.h)

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_mg_destroy(self.h)
            self.h = None

    def shape(self, lev=1):
        s = np.zeros(3, dtype=np.int32)
        lib().orc_mg_shape(self.h, lev, s.ctypes.data)
        return tuple(int(v) for v in s)

    def get(self, ivar, lev=1):
        a = np.zeros(self.shape(lev))
        lib().orc_mg_get(self.h, lev, ivar, a.ctypes.data)
        return a

    def set(self, ivar, a, lev=1):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == self.shape(lev)
        lib().orc_mg_set(self.h, lev, ivar, a.ctypes.data)

    def params(self, tol=1e-6, maxite=20, omega=0.9):
        lib().orc_mg_params(self.h, tol, maxite, omega)

    def solve(self):
        n = ctypes.c_int(0)
        r = ctypes.c_double(0)
        lib().orc_mg_solve(self.h, ctypes.byref(n), ctypes.byref(r))
        return n.value, r.value


# ------------------------------------------------------------------ whole model
class OracleModel:
    """One subdomain of the LES model (core/model_les.py) on the CPU.

    ``desc`` holds: nx, ny, nz, nh, geometry, n_tracers, modelname, timestepping,
    dx, dy, dz, idx2, idy2, idz2, fparam, visc (None = off), and optionally
    tracer_diffusion = {"b": kappa, "t0": kappa, ...} for the opt-in tracer diffusion
    on the last stage (core/tracer.py:74-76; never applied by the reference's rhs), and
    tracer_order = 1..5 for the linear advection branch (0 = WENO, the reference),
    vf_order = 1..5 for the linear vortex-force branch (0 = WENO, the reference).
    modelname "advection" is core/model_advection.py.
    """

    def __init__(self, desc):
        self.desc = dict(desc)
        g = desc["geometry"]
        per = (1 if "x" in g else 0) | (2 if "y" in g else 0) | (4 if "z" in g else 0)
        self.per = per
        visc = desc.get("visc")
        self.h = lib().orc_model_create(
            desc["nx"], desc["ny"], desc["nz"], desc.get("nh", 3), per,
            desc.get("n_tracers", 0), MODELS[desc.get("modelname", "LES")],
            SCHEMES[desc.get("timestepping", "RK3_SSP")],
            desc["dx"], desc["dy"], desc["dz"], desc["idx2"], desc["idy2"], desc["idz2"],
            desc.get("fparam", 0.0), visc or 0.0, 1 if visc else 0, MG_TOPOLOGY[g])
        nh = desc.get("nh", 3)
        self.shape = (desc["nz"] + (2 * nh if per & 4 else 0),
                      desc["ny"] + (2 * nh if per & 2 else 0),
                      desc["nx"] + (2 * nh if per & 1 else 0))
        self.ntr = desc.get("n_tracers", 0)
        trd = desc.get("tracer_diffusion") or {}
        if trd:
            names = ["b"] + ["t%d" % k for k in range(self.ntr)]
            kappa = (ctypes.c_double * 9)()
            mask = 0
            for q, name in enumerate(names):
                if name in trd:
                    kappa[q] = float(trd[name])
                    mask |= 1 << q
            lib().orc_model_set_tracer_diffusion(self.h, kappa, mask)
        if desc.get("tracer_order", 0):
            lib().orc_model_set_tracer_order(self.h, int(desc["tracer_order"]))
        if desc.get("vf_order", 0):
            lib().orc_model_set_vf_order(self.h, int(desc["vf_order"]))

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_model_destroy(self.h)
            self.h = None

    def field(self, name):
        """numpy view (no copy) of a state field in (z, y, x) order."""
        if name.startswith("t") and name[1:].isdigit():
            fid = 14 + int(name[1:])
        else:
            fid = FIELDS[name]
        ptr = lib().orc_model_field(self.h, fid)
        n = int(np.prod(self.shape))
        return np.ctypeslib.as_array(ptr, shape=(n,)).reshape(self.shape)

    def register(self, r, q):
        ptr = lib().orc_model_reg(self.h, r, q)
        if not ptr:
            raise IndexError("register %d, prognostic %d out of range" % (r, q))
        n = int(np.prod(self.shape))
        return np.ctypeslib.as_array(ptr, shape=(n,)).reshape(self.shape)

    def mg_params(self, tol=1e-6, maxite=20, omega=0.9):
        lib().orc_model_mg_params(self.h, tol, maxite, omega)

    def mg_stats(self):
        n = ctypes.c_int(0)
        r = ctypes.c_double(0)
        lib().orc_model_mg_stats(self.h, ctypes.byref(n), ctypes.byref(r))
        return n.value, r.value

    def diagnose(self):
        lib().orc_model_diagnose(self.h)

    def vortex_force(self, reg=0):
        """register `reg` = vortex force only (core/vortex_force.py:69-81)"""
        lib().orc_model_vortex_force(self.h, reg)

    def vfwork(self, box):
        """vortex-force work into field `work` and its sum over `box` = (k0, k1, j0, j1,
        i0, i1) (core/online_diag.py:11-35)"""
        b = np.ascontiguousarray(box, dtype=np.int64)
        return lib().orc_model_vfwork(self.h, b.ctypes.data)

    def project(self):
        """Advection.make_u_divergentfree (core/model_advection.py:38-53)"""
        lib().orc_model_project(self.h)

    def rhs(self, reg=0, last=False):
        lib().orc_model_rhs(self.h, reg, 1 if last else 0)

    def forward(self, t, dt):
        lib().orc_model_forward(self.h, float(t), float(dt))

    def set_forcing(self, fn):
        """fn(reg, t) adds tendencies into register set `reg` (numpy views from
        `register`) after each right-hand side; None detaches it."""
        if fn is None:
            self._forcing_cb = None
            lib().orc_model_set_forcing(self.h, None, None)
            return
        proto = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_void_p)
        self._forcing_cb = proto(lambda user, reg, t, stream: fn(reg, t))
        lib().orc_model_set_forcing(self.h, ctypes.cast(self._forcing_cb, ctypes.c_void_p), None)

    def fill(self, name):
        lib().orc_model_fill(self.h, FIELDS[name])

    def compute_dt(self, auto_dt, dt0, cfl, dt_max):
        """core/nyles.py:227-260"""
        if not auto_dt:
            return dt0
        umax = np.sqrt(lib().orc_model_max_U2(self.h))
        if umax == 0.0:
            return dt_max
        return min(cfl / umax, dt_max)
