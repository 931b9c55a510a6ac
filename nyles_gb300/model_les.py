"""LES model of one subdomain on the GPU.

Interface of the reference's core/model_les.py:33-175 (and of the Euler3d and linear
variants, core/model_les_euler.py and core/nyles.py:92-100): ``LES(param, grid,
linear=False)`` with ``state``, ``timescheme``, ``forward(t, dt) -> blowup``,
``rhs(state, t, dstate, last=False)`` and ``diagnose_var(state)``.

All arithmetic runs in libnyles_gb300.so; this class owns the device arrays (torch
tensors) and passes their pointers through the C ABI.
"""
import ctypes

import torch

from . import _native as nat
from . import timescheme as ts
from . import variables as var


def make_desc(param, grid, modelname):
    """NylesDesc of a parameter dictionary (one subdomain)."""
    geometry = param["geometry"]
    d = nat.NylesDesc()
    d.nx, d.ny, d.nz, d.nh = param["nx"], param["ny"], param["nz"], param["nh"]
    d.periodic_x = int("x" in geometry)
    d.periodic_y = int("y" in geometry)
    d.periodic_z = int("z" in geometry)
    d.n_tracers = param.get("n_tracers", 0)
    d.model = nat.MODEL[modelname]
    diff = param.get("diff_coef", {}) or {}
    d.add_viscosity = int("u" in diff)
    d.viscosity = float(diff.get("u", 0.0))
    # tracer diffusion (core/tracer.py:74-76): live in the advection model, whose rhs
    # passes `last` (core/model_advection.py:59-61); in LES only with the gpu parameter
    # tracer_diffusion (the reference's LES.rhs never applies it)
    gpu = param.get("gpu", {}) or {}
    if modelname == "advection" or gpu.get("tracer_diffusion", False):
        for q, name in enumerate(["b"] + ["t%d" % k for k in range(d.n_tracers)]):
            if name in diff:
                d.tracer_diffusivity[q] = float(diff[name])
                d.tracer_diffusion |= 1 << q
    # tracer_scheme "linear": the orderA interpolation of the linear branch of
    # core/fortran_upwind.f90:32-61 instead of WENO (the reference hard-codes WENO)
    if gpu.get("tracer_scheme", "weno") == "linear":
        d.tracer_order = int(param.get("orderA", 5))
    # vf_scheme "linear": the orderVF interpolation of the linear branch of
    # core/fortran_vortex_force.f90:43-55,121-133 instead of WENO (hard-coded there)
    if gpu.get("vf_scheme", "weno") == "linear":
        d.vf_order = int(param.get("orderVF", 5))
    d.dx, d.dy, d.dz = grid.dx, grid.dy, grid.dz
    d.idx2, d.idy2, d.idz2 = grid.idx2, grid.idy2, grid.idz2
    d.dx2 = grid.dx ** 2
    # covariant Coriolis parameter (core/model_les.py:61-67)
    d.fparam = float(param["coriolis"] * (grid.dx * grid.dy)) if param.get("rotating", False) else 0.0
    return d


# mixed precision, mg_krylov "auto": FCG at squared residual ratios at or below this
# (relative residual 1e-8)
KRYLOV_AUTO_TOL = 1e-16
# mg_warm_start modes (nyles_model_set_mg_warm_start; each needs the arrays of the ones
# before it and more) and the one "auto" takes with FCG
WARM_STARTS = {"last": 0, "stage": 1, "extrapolate": 2, "extrapolate2": 3, "extrapolate3": 4, "auto": None}
WARM_AUTO = "extrapolate2"


def warm_start_mode(warm, precision, krylov_on):
    """nyles_model_set_mg_warm_start mode of the gpu parameter mg_warm_start"""
    if warm not in WARM_STARTS:
        raise ValueError("mg_warm_start must be one of %s" % ", ".join(WARM_STARTS))
    if warm not in ("auto", "last") and precision == "fp64":
        raise ValueError("mg_warm_start = '%s' needs the mixed precision (the FP64 solve keeps the "
                         "reference's warm start)" % warm)
    if warm == "auto":
        warm = WARM_AUTO if krylov_on else "last"
    return WARM_STARTS[warm]


def krylov_on(krylov, precision, tol):
    """whether the mixed solve runs FCG for the gpu parameter mg_krylov at tolerance tol"""
    if krylov not in ("auto", "on", "off"):
        raise ValueError("mg_krylov must be 'auto', 'on' or 'off'")
    if precision == "fp64":
        if krylov == "on":
            raise ValueError("mg_krylov = 'on' needs the mixed precision (the FP64 solve keeps the reference's "
                             "iteration)")
        return False
    return krylov == "on" or (krylov == "auto" and float(tol) <= KRYLOV_AUTO_TOL)


def creation_warm_mode(gpu, precision):
    """warm start mode whose arrays a new model's workspace holds: the one its
    parameters select"""
    return warm_start_mode(gpu.get("mg_warm_start", "auto"), precision,
                           krylov_on(gpu.get("mg_krylov", "auto"), precision, gpu.get("mg_tol", 1e-6)))


class LES(object):
    """One subdomain of the LES / Euler3d / linear model on cuda:0 (or `device`)."""

    modelname = "LES"

    def __init__(self, param, grid, linear=False, device=None, arena=None):
        if not torch.cuda.is_available():
            raise RuntimeError("nyles_gb300 needs a CUDA GPU: the model runs only through libnyles_gb300.so")
        self.lib = nat.lib()
        if linear:
            self.modelname = "linear"
        self.nonlinear = not linear
        self.grid = grid
        self.param = param
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        gpu = param.get("gpu", {}) if isinstance(param.get("gpu"), dict) else {}
        self.precision = param.get("precision", gpu.get("precision", "fp64"))
        self.dtype = torch.float64 if self.precision == "fp64" else torch.float32
        ntr = param.get("n_tracers", 0)
        if ntr > nat.MAX_TRACERS:
            raise ValueError("at most %d tracers" % nat.MAX_TRACERS)
        self.traclist = ["b"] + var.tracer_names(ntr) if self.modelname != "Euler3d" else [""] + var.tracer_names(ntr)
        self.state = var.get_state(param, dtype=self.dtype, device=self.device, arena=arena)
        self.neighbours = param["neighbours"]
        self.orderA = param.get("orderA", 5)
        self.orderVF = param.get("orderVF", 5)
        self.orderKE = param.get("orderKE", 2)
        self.rotating = param.get("rotating", False)
        self.forced = param.get("forced", False)
        self.diff_coef = param.get("diff_coef", {}) or {}
        self.add_viscosity = "u" in self.diff_coef
        if self.add_viscosity:
            self.viscosity = self.diff_coef["u"]
        self.fparameter = param["coriolis"] * grid.dx * grid.dy if self.rotating else 0.0
        self.desc = make_desc(param, grid, self.modelname)
        self.timescheme = ts.Timescheme(param, self.state, model=self, arena=arena)
        self.timescheme.set(self.rhs, self.diagnose_var)
        # native model: arrays owned here, pointers bound once
        h = ctypes.c_void_p()
        nat.check(self.lib.nyles_model_create(ctypes.byref(self.desc), nat.SCHEME[param["timestepping"]],
                                              nat.PRECISION[self.precision], ctypes.byref(h)))
        self._h = h
        # the workspace holds the arrays of the warm start the parameters select
        self._warm_alloc = creation_warm_mode(gpu, self.precision)
        nat.check(self.lib.nyles_model_set_mg_warm_start(h, self._warm_alloc))
        nbytes = ctypes.c_size_t()
        nat.check(self.lib.nyles_model_workspace_bytes(h, ctypes.byref(nbytes)))
        if arena is not None:
            self.workspace = arena.take((nbytes.value,), torch.uint8)
            ws, off = self.workspace.data_ptr(), 0
        else:
            self.workspace = torch.zeros(nbytes.value + 256, dtype=torch.uint8, device=self.device)
            ws = self.workspace.data_ptr()
            ws = (ws + 255) & ~255
            off = ws - self.workspace.data_ptr()
        self._ws_used = self.workspace[off:off + nbytes.value]   # the aligned bytes the library uses
        self._fields = nat.ptr_array([s.data_ptr() for s in self.state.scalars()])
        self._regs = nat.ptr_array(self.timescheme.register_pointers())
        nat.check(self.lib.nyles_model_bind(h, self._fields, self._regs, ctypes.c_void_p(ws)))
        self.set_mg_params(gpu.get("mg_tol", 1e-6), gpu.get("mg_maxite", 20), gpu.get("mg_omega", 0.9),
                           krylov=gpu.get("mg_krylov", "auto"), warm_start=gpu.get("mg_warm_start", "auto"))
        self.stats = []
        # graph replay of fixed-dt steps (see forward)
        self.use_graphs = bool(gpu.get("graphs", True))
        self.graph = None
        self._last_dt = None
        self._first_step_pending = param["timestepping"] == "LFAM3"
        self._profiling = False
        self._forcing_cb = None
        self._forcing_error = None
        self.forcing = None

    # ------------------------------------------------------------------ user forcing
    @property
    def forcing(self):
        """User forcing (core/model_les.py:143-144): an object with
        `add(state, dstate, t)` that adds its tendencies into `dstate` with device tensor
        operations; it is called after every right-hand side when the parameter
        `forced` is set. Forced steps are never replayed from a graph."""
        return self._forcing

    @forcing.setter
    def forcing(self, f):
        self._forcing = f
        if self.forced and f is not None:
            if self.graph is not None:
                self.release_graph()

            def call(user, reg, t, stream):
                try:
                    if stream:
                        with torch.cuda.stream(torch.cuda.ExternalStream(stream, device=self.device)):
                            f.add(self.state, self.timescheme.registers[reg], t)
                    else:
                        f.add(self.state, self.timescheme.registers[reg], t)
                except BaseException as e:   # raised again by forward(): nothing propagates through C
                    self._forcing_error = e

            self._forcing_cb = nat.FORCING_FN(call)
            nat.check(self.lib.nyles_model_set_forcing(self._h, ctypes.cast(self._forcing_cb, ctypes.c_void_p), None))
        else:
            self._forcing_cb = None
            nat.check(self.lib.nyles_model_set_forcing(self._h, None, None))

    def _raise_forcing_error(self):
        e, self._forcing_error = self._forcing_error, None
        if e is not None:
            raise e

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self.lib.nyles_model_destroy(h)
            except Exception:
                pass
            self._h = None

    # ------------------------------------------------------------------ settings
    def set_mg_params(self, tol=1e-6, maxite=20, omega=0.9, krylov=None, warm_start=None):
        """Multigrid stop rule: sum(r^2)/sum(b^2) < tol or maxite V-cycles. `krylov`
        ("auto", "on", "off"; None keeps the current mode) selects the mixed-precision
        solver: FCG(1) preconditioned by the V-cycle, or the reference's stationary
        iteration; "auto" takes FCG when tol <= KRYLOV_AUTO_TOL, where both solvers land
        within the tolerance of the exact solution (at looser tolerances the stationary
        iterates are the ones that track the FP64 solve). `warm_start` ("auto", "stage",
        "extrapolate", "last"; None keeps the current mode) picks the start of each
        solve: the previous solve's solution (the reference's), or, mixed precision only,
        the solution of the same stage one step earlier, or its linear extrapolation from
        the same stage's last two (three, four: "extrapolate2", "extrapolate3")
        solutions; "auto" takes WARM_AUTO exactly when FCG runs, for the same reason, and
        no more than the workspace holds (the mode the model was created with). A
        captured graph holds the solver and its parameters, so it is released first."""
        if getattr(self, "graph", None) is not None:
            self.release_graph()
        if krylov is not None:
            if krylov not in ("auto", "on", "off"):
                raise ValueError("mg_krylov must be 'auto', 'on' or 'off'")
            self.mg_krylov = krylov
        mode = getattr(self, "mg_krylov", "auto")
        nat.check(self.lib.nyles_model_set_mg_params(self._h, float(tol), int(maxite), float(omega)))
        use = krylov_on(mode, self.precision, tol)
        nat.check(self.lib.nyles_model_set_mg_krylov(self._h, 1 if use else 0))
        self.krylov = use
        if warm_start is not None:
            warm_start_mode(warm_start, self.precision, use)      # validates
            self.mg_warm_start = warm_start
        wanted = getattr(self, "mg_warm_start", "auto")
        code = warm_start_mode(wanted, self.precision, use)
        if wanted == "auto":
            code = min(code, self._warm_alloc)
        elif code > self._warm_alloc:
            raise ValueError("mg_warm_start = '%s' needs arrays this model's workspace does not hold: pass it in "
                             "the parameters the model is created with" % wanted)
        nat.check(self.lib.nyles_model_set_mg_warm_start(self._h, code))
        self.warm_mode = next(k for k, v in WARM_STARTS.items() if v == code)
        self.warm_per_stage = code > 0

    def mg_stats(self):
        s = nat.NylesMgStats()
        nat.check(self.lib.nyles_model_mg_stats(self._h, ctypes.byref(s)))
        return {"nite": s.nite, "res": s.res, "solves": s.solves, "vcycles": s.vcycles,
                "not_converged": s.not_converged, "nonfinite": s.nonfinite}

    def update_stats(self):
        """Append the multigrid statistics and max|div| of the state to `stats`
        (core/model_les.py:151-160; the reference's run loop does not call it)."""
        s = self.mg_stats()
        s["maxdiv"] = float(self.state.div.view().abs().max())
        self.stats.append(s)

    def write_stats(self, path):
        """Pickle `stats` to <path>/stats.pkl (core/model_les.py:162-164)."""
        import os
        import pickle
        with open(os.path.join(path, "stats.pkl"), "wb") as fid:
            pickle.dump(self.stats, fid)

    # ------------------------------------------------------------------ model API
    def _check_state(self, state):
        if state is not self.state:
            raise NotImplementedError("the GPU model advances its own state (model.state) only")

    def diagnose_var(self, state):
        """Halo fill, projection, vorticity and kinetic energy (core/model_les.py:98-127)."""
        self._check_state(state)
        nat.check(self.lib.nyles_model_diagnose(self._h, nat.stream_ptr()))

    def rhs(self, state, t, dstate, last=False):
        """Right-hand side into `dstate` (core/model_les.py:130-144)."""
        self._check_state(state)
        fields = nat.ptr_array([s.data_ptr() for s in state.scalars()])
        ds = nat.ptr_array([s.data_ptr() for s in dstate.scalars()])
        fn = self.lib.nyles_rhs_f64 if self.precision == "fp64" else self.lib.nyles_rhs_f32
        nat.check(fn(ctypes.byref(self.desc), fields, ds, 1 if last else 0, nat.stream_ptr()))
        if self.forced:
            self._require_forcing()
            self.forcing.add(state, dstate, t)

    def _require_forcing(self):
        if self._forcing is None:
            raise RuntimeError("the parameter `forced` is set but no forcing is attached (model.forcing = ...)")

    def forward(self, t, dt):
        """One time step (core/model_les.py:147-149). Returns the blow-up flag: True
        when a pressure solve of an eagerly run step met a non-finite divergence (the
        reference's flag is never set). Replayed steps return False; Nyles.run checks
        them with the CFL reduction.

        With graphs on (gpu parameter `graphs`), the second consecutive call with the same
        dt captures the step into a CUDA graph, and every later call with that dt replays
        it: the same kernels, with the multigrid stop test on the device instead of one
        host round trip per V-cycle. A call with another dt runs eagerly."""
        if self.forced:
            self._require_forcing()
        dt = float(dt)
        if self.use_graphs and not self._profiling and not self._first_step_pending and not self.forced:
            if self.graph == (dt, 1):
                self.replay()
                return False
            if self._last_dt == dt:
                self.capture_graph(dt, 1)
                self.replay()
                return False
        self._last_dt = dt
        rc = self.lib.nyles_model_forward(self._h, float(t), dt, nat.stream_ptr())
        self._raise_forcing_error()
        self._first_step_pending = False
        if rc == nat.NYLES_BLOWUP:   # a projection met a non-finite divergence
            return True
        nat.check(rc)
        return False

    def profile(self, enable=True):
        """Per-phase CUDA-event timing of eager steps (graph replay is off meanwhile)."""
        self._profiling = bool(enable)
        nat.check(self.lib.nyles_model_profile(self._h, 1 if enable else 0))

    def capture_graph(self, dt, nsteps=1):
        """Record `nsteps` time steps with fixed `dt` into one CUDA graph (the multigrid
        stop test runs on the device). LFAM3 must have taken its first step."""
        nat.check(self.lib.nyles_model_capture(self._h, float(dt), int(nsteps)))
        self.graph = (float(dt), int(nsteps))

    def replay(self, stream=None):
        """Launch the captured graph: advances the state by its `nsteps` steps."""
        nat.check(self.lib.nyles_model_graph_launch(self._h, nat.stream_ptr(stream)))

    def release_graph(self):
        nat.check(self.lib.nyles_model_graph_release(self._h))
        self.graph = None

    def max_U2(self):
        """max of U^2+V^2+W^2 over the arrays; raises BlowUp on a non-finite value."""
        out = ctypes.c_double()
        nat.check(self.lib.nyles_model_max_U2(self._h, ctypes.byref(out), nat.stream_ptr()))
        return out.value

    def snapshot(self):
        """Host copy of everything a continued run depends on: all state fields, the
        time-scheme registers, the multigrid workspace (warm-started solution) and the
        LFAM3 first-step flag. `restore` on a model built from the same parameters
        continues bit for bit."""
        torch.cuda.synchronize(self.device)
        first = ctypes.c_int()
        nat.check(self.lib.nyles_model_get_first_step(self._h, ctypes.byref(first)))
        return {"state": self.state.storage.cpu(), "registers": self.timescheme.storage.cpu(),
                "workspace": self._ws_used.cpu(), "first_step": first.value}

    def restore(self, snap):
        for key, dst in (("state", self.state.storage), ("registers", self.timescheme.storage),
                         ("workspace", self._ws_used)):
            src = snap[key]
            if tuple(src.shape) != tuple(dst.shape) or src.dtype != dst.dtype:
                raise ValueError("snapshot %s does not match this model (%s %s vs %s %s)"
                                 % (key, tuple(src.shape), src.dtype, tuple(dst.shape), dst.dtype))
            dst.copy_(src)
        nat.check(self.lib.nyles_model_set_first_step(self._h, int(snap["first_step"])))
        self._first_step_pending = bool(snap["first_step"])
        self._last_dt = None
        torch.cuda.synchronize(self.device)

    def reset_timescheme(self):
        nat.check(self.lib.nyles_model_reset_scheme(self._h))
        self._first_step_pending = self.param["timestepping"] == "LFAM3"
        self._last_dt = None


class Euler3d(LES):
    """Euler equations without buoyancy (core/model_les_euler.py)."""

    modelname = "Euler3d"

    def __init__(self, param, grid, device=None, arena=None):
        if param["geometry"] not in ("closed", "perio_xyz"):
            # core/model_les_euler.py:80-90 maps only closed and perio_xyz to a multigrid topology
            raise ValueError("Euler3d supports the geometries closed and perio_xyz")
        super().__init__(param, grid, linear=False, device=device, arena=arena)
