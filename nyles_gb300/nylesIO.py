"""History files of a run (the interface of the reference's core/nylesIO.py:82-618).

``NylesIO(param)`` resolves the output directory and file names from `datadir`,
`expname` and `mode` ("overwrite", "count"; "continue" is refused as in the reference),
``init(state, grid, t, n)`` creates the history file with the reference's dimensions,
coordinates, variable names, long names, units and parameter attributes and writes the
first frame, and ``write(state, t, n)`` appends a frame every `timestep_history`.

The file is netCDF classic (64-bit offset), readable by the same netCDF tools as the
reference's files; each frame is one record appended in place (ncwriter.ClassicWriter).
Writing is asynchronous: each frame is copied from the device into pinned host buffers
on the current CUDA stream (so later steps cannot overtake the copy) and a background
thread waits for the copy and appends it to the file; ``flush()`` waits for all pending
frames.
"""
import os
import queue
import shutil
import threading

import numpy as np
import torch

from .ncwriter import ClassicWriter

MAX_LENGTH_ATTRIBUTE = 100


class NylesIO(object):
    def __init__(self, param):
        self.disk_limit = param["disk_space_warning"]
        self.simplified_grid = param["simplified_grid"]
        self.variables_in_history = param["variables_in_history"]
        self.dt_hist = param["timestep_history"]
        self.include_halo = param["include_halo"]
        self.t_next_hist = 0.0
        self.n_hist = 0
        self.last_saved_frame = None
        self.myrank = param.get("myrank", 0)
        self.unitT = param["unit_duration"]
        self.unitL = param["unit_length"]
        self.n_tracers = param.get("n_tracers", 0)
        self.experiment_parameters = self._attributes(param)
        datadir = os.path.expanduser(param["datadir"])
        expname = param["expname"]
        out_dir = os.path.join(datadir, expname)
        if param["mode"] == "count":
            counter = 0
            while True:
                full = "{}_{:04d}".format(expname, counter)
                out_dir = os.path.join(datadir, full)
                if not os.path.exists(out_dir):
                    break
                counter += 1
            expname = full
        elif param["mode"] == "continue":
            if not os.path.exists(out_dir):
                raise ValueError(
                    "cannot load experiment to continue: no directory exists with the name {!r}; please "
                    "specify a correct path or change the mode of the experiment.".format(out_dir))
            raise NotImplementedError("mode 'continue' (the reference does not implement it either); "
                                      "use LES.snapshot/restore to resume a run")
        elif param["mode"] != "overwrite":
            raise ValueError("unknown mode: {}".format(param["mode"]))
        self.hist_path = os.path.join(out_dir, expname + "_%02i" % self.myrank + "_hist.nc")
        self.script_path = os.path.join(out_dir, expname + ".py")
        self.output_directory = out_dir
        os.makedirs(self.output_directory, exist_ok=True)
        self._queue = None
        self._thread = None
        self._error = None

    # ------------------------------------------------------------------ helpers
    @staticmethod
    def _attributes(param):
        """Parameters as netCDF attributes: numbers and strings as they are, booleans as
        "True"/"False", anything else as "<type>: repr" cut to MAX_LENGTH_ATTRIBUTE."""
        out = {}
        for key, value in param.items():
            if isinstance(value, bool):
                out[key] = str(value)
            elif isinstance(value, (int, float, str)):
                out[key] = value
            else:
                s = "{}: {}".format(type(value), repr(value))[:MAX_LENGTH_ATTRIBUTE + 1]
                if len(s) > MAX_LENGTH_ATTRIBUTE:
                    s = s[:MAX_LENGTH_ATTRIBUTE - 3] + "..."
                out[key] = s
        return out

    def unit(self, dimensions):
        """Units of a dimension string ("L.T^-1" -> "m s-1")."""
        units = dimensions
        for k, v in {"T": self.unitT, "L": self.unitL, "^": "", ".": " "}.items():
            units = units.replace(k, v)
        return units

    # ------------------------------------------------------------------ file creation
    def init(self, state, grid, t=0.0, n=0):
        toc = state.toc
        if self.variables_in_history == "all":
            names = list(toc.keys())
        elif self.variables_in_history == "prognostic":
            names = state.get_prognostic_variables()
        elif self.variables_in_history == "p+p":
            names = state.get_prognostic_variables()
            if "p" not in toc:
                raise ValueError("pressure is not a variable of this model; please change the parameter "
                                 "variables_in_history.")
            names.append("p")
        else:
            names = list(self.variables_in_history)
            if any(v not in toc for v in names):
                raise ValueError("a variable chosen for the history file does not exist in this model.  "
                                 "The available variables are " + str(toc))
            for i in range(self.n_tracers):
                if "t%d" % i not in names:
                    names.append("t%d" % i)
        if not names:
            raise ValueError("no variables are selected for the history file.  This means, all calculation "
                             "results are lost.  I refuse to waste energy like this.")
        self.variables_in_history = names
        self.create_history_file(grid, [state.get(v) for v in names])
        self.write_history_file(state, t, n)
        self.t_next_hist = t + self.dt_hist

    def create_history_file(self, grid, variables):
        k0, k1, j0, j1, i0, i1 = grid.domainindices
        self.idx = {"x": slice(i0, i1), "y": slice(j0, j1), "z": slice(k0, k1)}
        dims = [("t", None)]
        points = ["b", "u", "v", "w", "vor_i", "vor_j", "vor_k"]
        for x, i in zip("xyz", "ijk"):
            if self.include_halo:
                size = grid.size[i]
                self.idx[x] = slice(None)
            else:
                size = getattr(grid, "n" + x)
            if self.simplified_grid:
                dims.append((x, size))
            else:
                for p in points:
                    dims.append(("{}_{}".format(x, p), size))
        ncvars = [("n", ("t",), "i4", {"long_name": "integration step in the model run"}),
                  ("t", ("t",), "f8", {"long_name": "time in the model run", "units": self.unit("T")})]
        fixed = {}
        # 1-D coordinates of each point family (core/grid.py:93-158)
        # (long names as the reference's grid variables: "x at cell faces y-component" is
        # the x coordinate of v-points)
        coords = {
            "b": ("x_b", "y_b", "z_b", grid.x_b_1D, grid.y_b_1D, grid.z_b_1D, "{} at cell centers"),
            "u": ("x_u", "y_u", "z_u", grid.x_u_1D, grid.y_u_1D, grid.z_u_1D, "{} at cell faces x-component"),
            "v": ("x_v", "y_v", "z_v", grid.x_v_1D, grid.y_v_1D, grid.z_v_1D, "{} at cell faces y-component"),
            "w": ("x_w", "y_w", "z_w", grid.x_w_1D, grid.y_w_1D, grid.z_w_1D, "{} at cell faces z-component"),
            "vor_i": ("x_vor_i", "y_vor_i", "z_vor_i", grid.x_vor_i_1D, grid.y_vor_i_1D, grid.z_vor_i_1D,
                      "{} at cell edges x-component"),
            "vor_j": ("x_vor_j", "y_vor_j", "z_vor_j", grid.x_vor_j_1D, grid.y_vor_j_1D, grid.z_vor_j_1D,
                      "{} at cell edges y-component"),
            "vor_k": ("x_vor_k", "y_vor_k", "z_vor_k", grid.x_vor_k_1D, grid.y_vor_k_1D, grid.z_vor_k_1D,
                      "{} at cell edges z-component"),
        }
        for p, (nx_, ny_, nz_, cx, cy, cz, longname) in coords.items():
            if self.simplified_grid and p != "b":
                continue
            for name, data, axis in ((nx_, cx, "x"), (ny_, cy, "y"), (nz_, cz, "z")):
                vname = axis if self.simplified_grid else name
                ncvars.append((vname, (vname,), "f8", {"long_name": longname.format(axis), "units": self.unit("L")}))
                fixed[vname] = np.asarray(data)[self.idx[axis]]
        self.hist_variables = {}

        def vdims(p):
            return ("t", "z", "y", "x") if self.simplified_grid else ("t", "z_" + p, "y_" + p, "x_" + p)

        def add(hist_name, p, var):
            ncvars.append((hist_name, vdims(p), "f8", {"long_name": var.name, "units": self.unit(var.dimension)}))
            self.hist_variables[hist_name] = var.nickname

        for var in variables:
            nature = var.get_nature()
            if nature == "scalar":
                add(var.nickname, "b", var)
            elif nature == "velocity":
                if var.nickname == "u":
                    modifier = str.lower
                elif var.nickname == "U":
                    modifier = str.upper
                else:
                    raise NotImplementedError("unknown kind of velocity: " + var.nickname)
                for i, u in zip("ijk", "uvw"):
                    add(modifier(u), u, var[i])
            elif nature == "vorticity":
                for i in "ijk":
                    add(var[i].nickname, "vor_" + i, var[i])
            else:
                raise ValueError("unknown nature", nature, "of variable", var.nickname)
        self.file = ClassicWriter(self.hist_path, dims, self.experiment_parameters, ncvars, fixed)

    # ------------------------------------------------------------------ frames
    def write(self, state, t, n):
        """Append a frame when t reaches the next history time. Returns True when the run
        should stop (never: a low-disk warning is printed instead of the reference's
        interactive pause)."""
        if t < self.t_next_hist:
            return False
        self.write_history_file(state, t, n)
        self.t_next_hist += self.dt_hist
        if self.disk_limit > 0:
            try:
                st = os.statvfs(self.output_directory)
                free = st.f_frsize * st.f_bavail / 1e9
                if free < self.disk_limit:
                    print("\nWarning: only %.2f GB left on the disk of %s" % (free, self.output_directory))
            except OSError:
                self.disk_limit = 0
        return False

    def finalize(self, state, t, n):
        """Write the final state unless step n is already the last frame, then wait for
        every frame (core/nylesIO.py:336-346)."""
        if n != self.last_saved_frame:
            self.write_history_file(state, t, n)
        self.flush()

    def save_array_3D(self, data, name, description=""):
        """Add a (z, y, x) array of the simplified grid as a variable of the history file
        (core/nylesIO.py:348-363)."""
        self.flush()
        atts = {"long_name": description} if description else {}
        if hasattr(data, "detach"):
            data = data.detach().cpu().numpy()
        self.file.add_fixed(name, ("z", "y", "x"), "f8", atts, data)

    def write_history_file(self, state, t, n):
        """Copy the frame to pinned host memory on the current stream and queue it."""
        idx = (self.idx["z"], self.idx["y"], self.idx["x"])
        frame = {}
        for hist_name, nickname in self.hist_variables.items():
            src = state.get(nickname).view("i")[idx]
            if src.is_cuda:
                dst = torch.empty(src.shape, dtype=src.dtype, pin_memory=True)
                dst.copy_(src, non_blocking=True)
            else:
                dst = src.clone()
            frame[hist_name] = dst
        event = None
        if any(v.is_pinned() for v in frame.values()):
            event = torch.cuda.Event()
            event.record()
        self._start_writer()
        self._queue.put((self.n_hist, t, n, frame, event))
        self.n_hist += 1
        self.last_saved_frame = n

    def _start_writer(self):
        if self._thread is not None:
            return
        self._queue = queue.Queue(maxsize=2)   # at most two frames in host memory
        self._thread = threading.Thread(target=self._writer, daemon=True)
        self._thread.start()

    def _writer(self):
        while True:
            item = self._queue.get()
            if item is None:
                self._queue.task_done()
                return
            k, t, n, frame, event = item
            try:
                if event is not None:
                    event.synchronize()
                if k != self.file.numrecs:
                    raise RuntimeError("history frame {} arrives after {} frames".format(k, self.file.numrecs))
                values = {name: data.numpy() for name, data in frame.items()}
                values["t"] = t
                values["n"] = n
                self.file.append(values)
            except BaseException as e:   # reported by flush()
                self._error = e
            self._queue.task_done()

    def flush(self):
        """Wait until every queued frame is in the file."""
        if self._queue is not None:
            self._queue.join()
        if self._error is not None:
            e, self._error = self._error, None
            raise e

    def close(self):
        if self._thread is not None:
            self._queue.put(None)
            self._thread.join()
            self._thread = None
        self.flush()

    def backup_scriptfile(self, filename):
        shutil.copyfile(filename, self.script_path)
