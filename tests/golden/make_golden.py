"""Generate golden vectors by running the REFERENCE's own Python orchestration.

Run where a checkout of the reference exists (the tests themselves never need it).
The path of the reference's ``core`` directory comes from the first argument or from the
environment variable NYLES_REFERENCE_CORE:

    python tests/golden/make_golden.py <reference checkout>/core

The reference's Python modules (core/nyles.py, core/model_les.py,
core/timescheme.py, core/projection.py, core/mgfordriver.py, core/mpi/halo.py,
core/variables.py, core/grid.py, ...) are imported unchanged. The native pieces they
call cannot be built here (no Fortran compiler, no MPI), so they are provided as
stand-in modules:

* the f2py libraries (fortran_vortex_force, fortran_upwind, fortran_vorticity,
  fortran_kinenergy, fortran_bernoulli, fortran_dissipation) call the CPU oracle's
  restated kernels;
* ``mgmod``/``build`` (the ctypes binding of mgfor) call the oracle's mgfor
  restatement with the same set/get/solve protocol;
* ``mpi4py`` is a one-rank communicator whose persistent requests deliver
  self-messages by tag, so core/mpi/halo.py performs its real periodic copies;
* netCDF IO, plotting and the old Python multigrid are inert stubs.

The fixtures therefore pin everything the reference does in Python — array views and
transposes, halo fills, projection glue, time-scheme arithmetic, CFL — against the
oracle's C++ restatement of that orchestration. Outputs: ``tests/golden/*.npz`` and
``tests/golden/params_cases.json``.
"""
import json
import os
import sys
import tempfile
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
REF = None   # the reference's core/ directory, set by main()
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle  # noqa: E402


# ------------------------------------------------------------------ stand-in modules
def _install_stubs():
    # f2py kernels -> oracle kernels (the `order` argument is ignored by the
    # reference, whose `linear` flag is hard-wired to .false.)
    m = types.ModuleType("fortran_vortex_force")
    m.vortex_force_direc = lambda U, vort, res, order: oracle.vortex_force_direc(U, vort, res)
    m.vortex_force_flip = lambda U, vort, res, order: oracle.vortex_force_flip(U, vort, res)
    sys.modules[m.__name__] = m
    m = types.ModuleType("fortran_upwind")
    m.upwind = lambda trac, u, dtrac, order: oracle.upwind(trac, u, dtrac)
    sys.modules[m.__name__] = m
    m = types.ModuleType("fortran_vorticity")
    m.vorticity = lambda ui, uj, wk: oracle.vorticity(ui, uj, wk)
    sys.modules[m.__name__] = m
    m = types.ModuleType("fortran_kinenergy")
    m.kin = lambda u, v, ke, ds2, order: oracle.kin(u, ke, ds2)
    sys.modules[m.__name__] = m
    m = types.ModuleType("fortran_bernoulli")
    m.gradke = lambda ke, du: oracle.gradke(ke, du)
    m.gradkeandb = lambda ke, b, du, dz: oracle.gradkeandb(ke, b, du, dz)
    m.div = lambda d, u, iflag: oracle.div(d, u, iflag)
    sys.modules[m.__name__] = m
    m = types.ModuleType("fortran_dissipation")
    m.add_laplacian = lambda phi, dphi, coef: oracle.add_laplacian(phi, dphi, coef)
    sys.modules[m.__name__] = m

    # one-rank MPI with persistent self-messages
    mpi = types.ModuleType("mpi4py")
    MPI = types.ModuleType("mpi4py.MPI")

    class _Req:
        mailbox = {}

        def __init__(self, buf, tag, send):
            self.buf, self.tag, self.send = buf, tag, send

    class _Comm:
        def Get_rank(self):
            return 0

        def Get_size(self):
            return 1

        def Send_init(self, buf, dest, tag=0):
            return _Req(buf, tag, True)

        def Recv_init(self, buf, source, tag=0):
            return _Req(buf, tag, False)

        def allreduce(self, x, op=None):
            return x

        def barrier(self):
            pass

        def Abort(self):
            raise SystemExit(1)

    class _Prequest:
        @staticmethod
        def Startall(reqs):
            for r in reqs:
                if r.send:
                    _Req.mailbox[r.tag] = r.buf.copy()

        @staticmethod
        def Waitall(reqs):
            for r in reqs:
                if not r.send:
                    r.buf[...] = _Req.mailbox.pop(r.tag)

    MPI.COMM_WORLD = _Comm()
    MPI.Prequest = _Prequest
    MPI.SUM, MPI.MAX = "sum", "max"
    mpi.MPI = MPI
    sys.modules["mpi4py"] = mpi
    sys.modules["mpi4py.MPI"] = MPI

    # mgfor ctypes binding -> oracle mgfor
    build = types.ModuleType("build")

    def ptr(thing):
        if isinstance(thing, (tuple, list)):
            return tuple(ptr(t) for t in thing)
        return thing
    build.ptr = ptr
    build.POINTER = lambda t: t
    build.c_int64 = int
    sys.modules["build"] = build

    mgmod = types.ModuleType("mgmod")
    MG_INSTANCES = []

    class _F:
        def __init__(self, fn):
            self.f = fn
            self.restype = None

        def __call__(self, *args):
            return self.f(*args)

    def get_ptrmg(npx, npy, nx, ny, nz, vertices, short, is3d, topology):
        assert npx == 1 and npy == 1 and is3d and not vertices
        h = oracle.OracleMG(nx, ny, nz, topology)
        h.params(*MG_PARAMS)
        MG_INSTANCES.append(h)
        return h

    def get_pyshape(h, lev, shape):
        s = h.shape(lev)
        shape[0], shape[1], shape[2] = s[0], s[1], s[2]

    def set_pyarray(h, lev, ivar, n1, n2, n3, x):
        h.set(ivar, x, lev)

    def get_pyarray(h, lev, ivar, n1, n2, n3, x):
        x[...] = h.get(ivar, lev)

    def solve(h):
        h.last = h.solve()

    funcs = {"get_ptrmg": get_ptrmg, "print_mginfos": lambda h: None, "solve": solve,
             "get_pyshape": get_pyshape, "set_pyarray": set_pyarray, "get_pyarray": get_pyarray}
    mgmod.get = lambda name, isfloat32=False: _F(funcs[name])
    mgmod.INSTANCES = MG_INSTANCES
    sys.modules["mgmod"] = mgmod

    # inert pieces (IO, plots, the superseded Python multigrid)
    for name in ("mg", "plotting", "matplotlib", "matplotlib.pyplot"):
        sys.modules[name] = types.ModuleType(name)
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    io = types.ModuleType("nylesIO")

    class NylesIO:
        def __init__(self, param):
            self.output_directory = tempfile.mkdtemp(prefix="nyles_golden_")
            self.hist_path = os.path.join(self.output_directory, "hist.nc")
            self.t_next_hist = 1e30
    io.NylesIO = NylesIO
    sys.modules["nylesIO"] = io
    return mgmod


MG_PARAMS = (1e-6, 20, 0.9)   # mg_types.f90:15-26 defaults


def _import_reference():
    for p in (REF, os.path.join(REF, "mpi")):
        if p not in sys.path:
            sys.path.insert(0, p)
    mgmod = _install_stubs()
    import parameters as refparams  # noqa
    import nyles as refnyles  # noqa
    return refparams, refnyles, mgmod


# ------------------------------------------------------------------ cases
CASES = [
    # name, geometry, modelname, scheme, (nx,ny,nz), L, n_tracers, auto_dt, dt, extras
    # isotropic box: with dx != dy or dz the reference's projection (p = x*dx**2,
    # core/mgfordriver.py:78) over-corrects and the run is unstable
    dict(name="closed_les_rk3", geometry="closed", modelname="LES", timestepping="RK3_SSP",
         n=(16, 8, 8), L=(2.0, 1.0, 1.0), n_tracers=0, auto_dt=False, dt=2e-3, steps=3, init="lock"),
    dict(name="perioxy_les_rk3_tracer", geometry="perio_xy", modelname="LES", timestepping="RK3_SSP",
         n=(8, 8, 8), L=(1.0, 1.0, 1.0), n_tracers=1, auto_dt=True, cfl=0.8, dt_max=0.05, steps=3, init="shear"),
    dict(name="perioxyz_euler_lfam3", geometry="perio_xyz", modelname="Euler3d", timestepping="LFAM3",
         n=(8, 8, 8), L=(6.283185307179586,) * 3, n_tracers=0, auto_dt=True, cfl=0.8, dt_max=0.4, steps=3, init="tgv"),
    dict(name="perioxyz_les_rk3", geometry="perio_xyz", modelname="LES", timestepping="RK3_SSP",
         n=(8, 8, 8), L=(6.283185307179586,) * 3, n_tracers=0, auto_dt=False, dt=5e-2, steps=2, init="tgv"),
    dict(name="closed_les_ef_rot_visc", geometry="closed", modelname="LES", timestepping="EF",
         n=(8, 8, 8), L=(1.0, 1.0, 1.0), n_tracers=0, auto_dt=False, dt=1e-3, steps=2, init="lock",
         rotating=True, coriolis=2.0, diff_coef={"u": 1e-3}),
    dict(name="perioxy_linear_lfam3", geometry="perio_xy", modelname="linear", timestepping="LFAM3",
         n=(8, 8, 8), L=(1.0, 1.0, 1.0), n_tracers=0, auto_dt=False, dt=1e-2, steps=3, init="shear"),
    # anisotropic grids (dx = 2 dy = 2 dz; dx = dz = dy / 2): three steps, before the
    # projection's over-correction grows large, pin p = x*dx**2 and the anisotropic metric
    dict(name="closed_les_rk3_aniso", geometry="closed", modelname="LES", timestepping="RK3_SSP",
         n=(16, 8, 8), L=(4.0, 1.0, 1.0), n_tracers=0, auto_dt=False, dt=2e-3, steps=3, init="lock"),
    dict(name="perioxy_les_rk3_2tracers_aniso", geometry="perio_xy", modelname="LES", timestepping="RK3_SSP",
         n=(16, 8, 16), L=(1.0, 1.0, 1.0), n_tracers=2, auto_dt=True, cfl=0.8, dt_max=0.05, steps=3, init="shear"),
    # 16^3: a multigrid of four levels (16, 8, 4, 2)
    dict(name="perioxy_les_lfam3_16", geometry="perio_xy", modelname="LES", timestepping="LFAM3",
         n=(16, 16, 16), L=(1.0, 1.0, 1.0), n_tracers=1, auto_dt=True, cfl=0.8, dt_max=0.05, steps=3, init="shear"),
    # Euler3d between walls (its projection precedes the halo fill) with a tracer; Euler
    # forward LES with a tracer in the triply periodic box
    dict(name="closed_euler_rk3_tracer", geometry="closed", modelname="Euler3d", timestepping="RK3_SSP",
         n=(16, 8, 8), L=(2.0, 1.0, 1.0), n_tracers=1, auto_dt=True, cfl=0.8, dt_max=0.05, steps=3, init="shear"),
    dict(name="perioxyz_les_ef_tracer", geometry="perio_xyz", modelname="LES", timestepping="EF",
         n=(8, 8, 8), L=(6.283185307179586,) * 3, n_tracers=1, auto_dt=False, dt=2e-2, steps=3, init="tgv"),
    # the linear model between walls, with viscosity
    dict(name="closed_linear_rk3_visc", geometry="closed", modelname="linear", timestepping="RK3_SSP",
         n=(16, 8, 8), L=(2.0, 1.0, 1.0), n_tracers=0, auto_dt=False, dt=2e-3, steps=3, init="lock",
         diff_coef={"u": 1e-3}),
]


def initial_state(case, grid, state, ntr, rng):
    """Seeded initial fields written the way experiment scripts do, through view('i')."""
    xb, yb, zb = grid.x_b.view("i"), grid.y_b.view("i"), grid.z_b.view("i")
    b = state.b.view("i")
    u = state.u["i"].view("i")
    v = state.u["j"].view("i")
    w = state.u["k"].view("i")
    if case["init"] == "lock":
        b[:] = np.where(xb < 0.5 * case["L"][0], -0.5, 0.5) + 1e-3 * rng.uniform(-1, 1, size=b.shape)
    elif case["init"] == "shear":
        zs = grid.z_vel["i"].view("i")
        u[:] = 0.1 * np.tanh((zs - 0.5) / 0.1) * grid.dx
        b[:] = zb.copy()
        v[:] += 1e-2 * rng.standard_normal(size=v.shape) * grid.dy
        w[:] += 1e-2 * rng.standard_normal(size=w.shape) * grid.dz
        for t in range(ntr):
            state.get("t%d" % t).view("i")[:] = np.tanh((zb - 0.5) / 0.1)
    elif case["init"] == "tgv":
        xu, yu, zu = grid.x_vel["i"].view("i"), grid.y_vel["i"].view("i"), grid.z_vel["i"].view("i")
        xv, yv, zv = grid.x_vel["j"].view("i"), grid.y_vel["j"].view("i"), grid.z_vel["j"].view("i")
        u[:] = np.sin(xu) * np.cos(yu) * np.cos(zu) * grid.dx
        v[:] = -np.cos(xv) * np.sin(yv) * np.cos(zv) * grid.dy
        u[:] += 1e-3 * rng.standard_normal(size=u.shape) * grid.dx
        v[:] += 1e-3 * rng.standard_normal(size=v.shape) * grid.dy
        w[:] += 1e-3 * rng.standard_normal(size=w.shape) * grid.dz
    # closed walls carry no normal velocity
    ngbs = state.b.param["neighbours"]
    if (0, 0, 1) not in ngbs:
        u[:, :, -1] = 0.0
    if (0, 1, 0) not in ngbs:
        v[:, -1, :] = 0.0
    if (1, 0, 0) not in ngbs:
        w[-1, :, :] = 0.0


def run_case(refparams, refnyles, mgmod, case, seed):
    refparams.InextensibleDict.frozen = False
    param = refparams.UserParameters()
    param.model["modelname"] = case["modelname"]
    param.model["geometry"] = case["geometry"]
    param.model["Lx"], param.model["Ly"], param.model["Lz"] = case["L"]
    param.model["n_tracers"] = case["n_tracers"]
    param.time["timestepping"] = case["timestepping"]
    param.time["auto_dt"] = case["auto_dt"]
    param.time["dt"] = case.get("dt", 0.1)
    param.time["cfl"] = case.get("cfl", 1.0)
    param.time["dt_max"] = case.get("dt_max", 1.0)
    param.physics["rotating"] = case.get("rotating", False)
    param.physics["coriolis"] = case.get("coriolis", 1.0)
    param.physics["diff_coef"] = case.get("diff_coef", {})
    nx, ny, nz = case["n"]
    param.discretization["global_nx"] = nx
    param.discretization["global_ny"] = ny
    param.discretization["global_nz"] = nz
    nyl = refnyles.Nyles(param)
    model = nyl.model
    state = model.state
    rng = np.random.Generator(np.random.PCG64(seed))
    initial_state(case, nyl.grid, state, case["n_tracers"], rng)
    progs = state.get_prognostic_scalars()
    out = {}
    for s in progs:
        out["init_" + s] = state.get(s).view("i").copy()
    model.diagnose_var(state)          # core/nyles.py:122
    mg = mgmod.INSTANCES[-1]
    out["nite_0"] = np.array(mg.last[0])
    t = 0.0
    dts = []
    nites = []
    for n in range(case["steps"]):
        dt = nyl.compute_dt()
        model.forward(t, dt)
        t += dt
        dts.append(dt)
        nites.append(mg.last[0])
    out["dts"] = np.array(dts)
    out["nites_last"] = np.array(nites)
    names = progs + ["p", "ke", "U_i", "U_j", "U_k", "vor_i", "vor_j", "vor_k", "div"]
    for s in names:
        out["final_" + s] = state.get(s).view("i").copy()
    # the reference's online diagnostic on the final state (core/online_diag.py:11-35)
    import online_diag
    diag = online_diag.VFwork(model, nyl.grid)
    diag.compute()
    out["vfwork_sum"] = np.array(diag.worksum)
    out["vfwork_work"] = state.work.view("i").copy()
    for c in "ijk":
        out["vfwork_du_" + c] = model.timescheme.dstate.u[c].view("i").copy()
    meta = dict(case)
    meta["seed"] = seed
    meta["dx"], meta["dy"], meta["dz"] = nyl.grid.dx, nyl.grid.dy, nyl.grid.dz
    meta["idx2"], meta["idy2"], meta["idz2"] = nyl.grid.idx2, nyl.grid.idy2, nyl.grid.idz2
    meta["fparam"] = float(model.fparameter)
    meta["nlevels"] = mg.nlevels
    out["meta"] = np.array(json.dumps(meta))
    return out


def params_cases(refparams):
    """Record what the reference's UserParameters.check() accepts and rejects."""
    cases = [
        ("model", "geometry", "open"), ("model", "Lx", -3), ("model", "Ly", "5"),
        ("IO", "expname", "foo/bar"), ("IO", "variables_in_history", "any"),
        ("IO", "timestep_history", -1.0), ("time", "cfl", 0), ("discretization", "global_nx", 5),
        ("discretization", "global_nx", 48), ("discretization", "global_nx", 96),
        ("discretization", "global_ny", 2 ** 60), ("MPI", "npx", 1.5), ("MPI", "nh", -1),
        ("discretization", "orderA", 4), ("discretization", "orderA", 6),
        ("time", "timestepping", "RK4"), ("model", "modelname", "Euler3d"),
        ("model", "n_tracers", -1), ("physics", "diff_coef", {"u": 1.0}),
        ("time", "auto_dt", 1), ("model", "Lz", 2),
    ]
    res = []
    for cat, key, value in cases:
        refparams.InextensibleDict.frozen = False
        p = refparams.UserParameters()
        getattr(p, cat)[key] = value
        try:
            p.check()
            res.append(dict(category=cat, key=key, value=value, error=None))
        except refparams.UserParameterError as e:
            res.append(dict(category=cat, key=key, value=value, error=str(e)))
    # npz larger than global_nz
    refparams.InextensibleDict.frozen = False
    p = refparams.UserParameters()
    p.discretization["global_nz"] = 1
    p.MPI["npz"] = 2
    try:
        p.check()
        err = None
    except refparams.UserParameterError as e:
        err = str(e)
    res.append(dict(category="MPI+discretization", key="npz>global_nz", value=[1, 2], error=err))
    # adding a new key is refused
    p = refparams.UserParameters()
    try:
        p.model["foo"] = 1
        err = None
    except refparams.UserParameterError as e:
        err = str(e)
    res.append(dict(category="model", key="foo", value=1, error=err, new_key=True))
    return res


def main(only=()):
    """Every case (or the named ones) and the parameter cases; a case's seed is fixed by
    its position in CASES."""
    refparams, refnyles, mgmod = _import_reference()
    os.makedirs(HERE, exist_ok=True)
    for k, case in enumerate(CASES):
        if only and case["name"] not in only:
            continue
        out = run_case(refparams, refnyles, mgmod, case, seed=100 + k)
        np.savez_compressed(os.path.join(HERE, case["name"] + ".npz"), **out)
        print("wrote", case["name"], "nites", out["nites_last"], "dts", out["dts"])
    with open(os.path.join(HERE, "params_cases.json"), "w") as f:
        json.dump(params_cases(refparams), f, indent=1)
    print("wrote params_cases.json")


if __name__ == "__main__":
    REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("NYLES_REFERENCE_CORE")
    if not REF or not os.path.isfile(os.path.join(REF, "nyles.py")):
        sys.exit("usage: make_golden.py <reference core/ directory> [case names] (or set NYLES_REFERENCE_CORE)")
    main(tuple(sys.argv[2:]))
