"""The Nyles driver: ``Nyles(param).run()`` for one subdomain on one GPU.

Interface of the reference's core/nyles.py:22-260: the constructor checks and freezes
the parameters, derives nx/ny/nz, the neighbours and the grid, and builds the model
(``LES``, ``Euler3d``, ``linear`` or ``advection``); ``run()`` projects the initial state and advances
it to ``tend`` with ``compute_dt()`` (CFL) and ``model.forward``, writing the netCDF
history file (nylesIO) when the gpu parameter `history` is on (the default).

Not part of this build: the interactive animation, and MPI decomposition (one subdomain
per process; npx = npy = npz = 1).
"""
import os
import pickle
import sys
import time

import numpy as np

from . import grid as grid_module
from . import model_advection
from . import model_les
from . import nylesIO
from . import online_diag
from . import topology as topo


def prepare_parameters(user_param):
    """Checked parameter dictionary of one subdomain (core/nyles.py:44-76): nx/ny/nz,
    the processor layout, neighbours and location, and the gpu category."""
    user_param.check()
    user_param.freeze()
    param = dict(user_param.view_parameters())
    param["gpu"] = dict(user_param.gpu)
    npx, npy, npz = param["npx"], param["npy"], param["npz"]
    if (npx, npy, npz) != (1, 1, 1):
        raise NotImplementedError("one subdomain per GPU: npx = npy = npz = 1 (no MPI in this build)")
    param["nx"] = param["global_nx"] // npx
    param["ny"] = param["global_ny"] // npy
    param["nz"] = param["global_nz"] // npz
    procs = [npz, npy, npx]
    loc = topo.rank2loc(0, procs)
    param["procs"] = procs
    param["myrank"] = 0
    param["neighbours"] = topo.get_neighbours(loc, procs, param["geometry"])
    param["loc"] = loc
    return param


def arena_bytes(user_param):
    """Bytes of the Arena (variables.Arena) that a Nyles model of these parameters
    carves its arrays from: the state, the time-scheme registers and the library's
    workspace, each 256-byte aligned."""
    import ctypes
    from . import _native as nat
    from . import variables as var
    param = prepare_parameters(user_param)
    grid = grid_module.Grid(param)
    size, _ = var.variable_shape(param)
    vol = int(size[0]) * int(size[1]) * int(size[2])
    prec = param["gpu"].get("precision", "fp64")
    es = 8 if prec == "fp64" else 4
    ntr = param.get("n_tracers", 0)
    desc = model_les.make_desc(param, grid, param["modelname"])
    h = ctypes.c_void_p()
    nat.check(nat.lib().nyles_model_create(ctypes.byref(desc), nat.SCHEME[param["timestepping"]],
                                           nat.PRECISION[prec], ctypes.byref(h)))
    try:
        nat.check(nat.lib().nyles_model_set_mg_warm_start(h, model_les.creation_warm_mode(param["gpu"], prec)))
        nb = ctypes.c_size_t()
        nat.check(nat.lib().nyles_model_workspace_bytes(h, ctypes.byref(nb)))
    finally:
        nat.lib().nyles_model_destroy(h)
    A = var.Arena.aligned
    return A((14 + ntr) * vol * es) + A(3 * (4 + ntr) * vol * es) + A(nb.value)


class Nyles(object):
    def __init__(self, user_param, device=None, arena=None):
        param = prepare_parameters(user_param)
        self.param = param
        self.myrank = param["myrank"]
        self.grid = grid_module.Grid(param)
        self.initiate(param, device, arena)

    def initiate(self, param, device=None, arena=None):
        """The model of `modelname` (core/nyles.py:92-100). `arena` (variables.Arena):
        carve the model's arrays from one buffer (batched serving)."""
        name = param["modelname"]
        if name == "LES":
            self.model = model_les.LES(param, self.grid, device=device, arena=arena)
        elif name == "Euler3d":
            self.model = model_les.Euler3d(param, self.grid, device=device, arena=arena)
        elif name == "linear":
            self.model = model_les.LES(param, self.grid, linear=True, device=device, arena=arena)
        elif name == "advection":
            self.model = model_advection.Advection(param, self.grid, device=device)
        else:
            raise NotImplementedError("modelname %r is not provided by the GPU build" % name)
        self.tend = param["tend"]
        self.auto_dt = param["auto_dt"]
        self.dt0 = param["dt"]
        self.cfl = param["cfl"]
        self.dt_max = param["dt_max"]
        self.blowup_check = param.get("gpu", {}).get("blowup_check", True)
        self.gridcellpersubdom = param["nx"] * param["ny"] * param["nz"]
        self.diag = online_diag.VFwork(self.model, self.grid)   # core/nyles.py:102
        # history files and param.pkl (core/nyles.py:78-87), unless the gpu parameter
        # `history` is off
        self.IO = None
        if param.get("gpu", {}).get("history", True):
            self.IO = nylesIO.NylesIO(param)
            with open(os.path.join(self.IO.output_directory, "param.pkl"), "wb") as fid:
                pickle.dump(param, fid)

    def compute_dt(self):
        """cfl / max|U| bounded by dt_max, or the fixed dt (core/nyles.py:227-260)."""
        if self.auto_dt:
            U_max = np.sqrt(self.model.max_U2())
            if U_max == 0.0:
                return self.dt_max
            return min(self.cfl / U_max, self.dt_max)
        return self.dt0

    def run(self, nsteps=None, verbose=True, callback=None):
        """Advance to tend (or `nsteps` steps). Returns (t, n, blowup).

        `callback(nyles, t, n)` is called after every step (e.g. for snapshots). At
        every history time (`timestep_history`) the vortex-force work is diagnosed and
        (t, Kdiss) appended to `self.kdiss` (core/nyles.py:166-171).
        """
        from . import _native as nat
        t, n = 0.0, 0
        dt_hist = float(self.param.get("timestep_history", 0.0))
        t_next_hist = dt_hist
        self.kdiss = []
        blowup = False
        try:
            self.model.diagnose_var(self.model.state)   # core/nyles.py:122
        except nat.BlowUp:
            blowup = True
        if self.IO is not None:                      # core/nyles.py:131-139
            if verbose:
                print("Creating output file:", self.IO.hist_path)
            self.IO.init(self.model.state, self.grid, t, n)
            t_next_hist = self.IO.t_next_hist
            script = sys.argv[0] if sys.argv else ""
            if script.endswith(".py") and os.path.isfile(script):
                if verbose:
                    print("Backing up script to:", self.IO.script_path)
                self.IO.backup_scriptfile(script)
        realtime0 = time.time()
        nonfinite_seen = self.model.mg_stats()["nonfinite"] if hasattr(self.model, "mg_stats") else 0
        while not blowup:
            try:
                dt = self.compute_dt()
            except nat.BlowUp:
                blowup = True
                if self.IO is not None:              # last frame at blow-up (core/nyles.py:186-201)
                    self.IO.t_next_hist = t
                    self.IO.write(self.model.state, t, n)
                break
            blowup = self.model.forward(t, dt)
            if not blowup and self.blowup_check and getattr(self.model, "graph", None) is not None:
                # a replayed step returns no flag: its solves count non-finite norms on the
                # device (one small read-back per step)
                nonfinite = self.model.mg_stats()["nonfinite"]
                blowup = nonfinite > nonfinite_seen
                nonfinite_seen = nonfinite
            t += dt
            n += 1
            if blowup:
                if self.IO is not None:
                    self.IO.t_next_hist = t
                    self.IO.write(self.model.state, t, n)
                break
            if t >= t_next_hist:                     # core/nyles.py:166-171
                Kdiss = self.diag.compute()
                self.kdiss.append((t, Kdiss))
                if verbose:
                    print(f"\nKdiss = {Kdiss}")
            if self.IO is not None:
                self.IO.write(self.model.state, t, n)
                t_next_hist = self.IO.t_next_hist
            elif t >= t_next_hist:
                t_next_hist += dt_hist
            if callback is not None:
                callback(self, t, n)
            if verbose:
                realtime = time.time()
                perf = (realtime - realtime0) / self.gridcellpersubdom
                realtime0 = realtime
                print("\rn = {:3d}, t = {:.2f}/{:.2f}, dt = {:.4f}, perf = {:.2e}".format(
                    n, t, self.tend, dt, perf), end="")
            if t >= self.tend or (nsteps is not None and n >= nsteps):
                break
        if self.blowup_check and not blowup:
            try:
                self.model.max_U2()
            except nat.BlowUp:
                blowup = True
        if self.IO is not None:                      # core/nyles.py:217-222
            self.IO.finalize(self.model.state, t, n)
            self.model.write_stats(self.IO.output_directory)
            if verbose:
                print("Output written to:", self.IO.hist_path)
        if verbose:
            print()
            print("BLOW UP!" if blowup else "Job completed as expected")
        return t, n, blowup
