"""Fields of the model: Scalar, Vector and State on device memory.

Interface of the reference's core/variables.py:52-437. The reference keeps each field
three times, once per orientation, and transposes on every change of orientation
(core/variables.py:146-182). Here each field is ONE row-major (z, y, x) array (the
reference's `view('i')` layout) inside a single state tensor, and the other
orientations are strided views of it — no copy, and writes through any view land in
the field:
    view('i') -> (z, y, x)   view('j') -> (x, z, y)   view('k') -> (y, x, z)
    flipview(d) puts direction d outermost.
"""
from collections import namedtuple

import torch

from . import topology as topo

ModelVariable = namedtuple("ModelVariable", ["type", "name", "dimension", "prognostic"])

# core/variables.py:38-47 (table-of-contents order = field ids of the C ABI)
modelvar = {
    "b": ModelVariable("scalar", "buoyancy", "L.T^-2", prognostic=True),
    "p": ModelVariable("scalar", "pressure", "L^2.T^-2", prognostic=False),
    "ke": ModelVariable("scalar", "kinetic energy", "L^2.T^-2", prognostic=False),
    "div": ModelVariable("scalar", "divergence", "T^-1", prognostic=False),
    "u": ModelVariable("velocity", "covariant velocity", "L^2.T^-1", prognostic=True),
    "U": ModelVariable("velocity", "contravariant velocity", "T^-1", prognostic=False),
    "vor": ModelVariable("vorticity", "vorticity", "L^2.T^-1", prognostic=False),
    "work": ModelVariable("scalar", "work", "L^2.T^-2", prognostic=False),
}

_PERM = {"i": (0, 1, 2), "j": (2, 0, 1), "k": (1, 2, 0)}
_FLIP = {"i": "j", "j": "k", "k": "i"}


def variable_shape(param):
    """(extents [nz, ny, nx] with halo, domainindices) of every field."""
    return topo.get_variable_shape([param["nz"], param["ny"], param["nx"]], param["neighbours"], param["nh"])


class Scalar(object):
    """A scalar field; `data` is a (z, y, x) tensor (a view into the state storage)."""

    def __init__(self, param, name, nickname, dimension, prognostic=False, data=None,
                 dtype=torch.float64, device="cpu"):
        self.param = {k: param[k] for k in ["nx", "ny", "nz", "nh", "neighbours"]}
        self.name = name
        self.nickname = nickname
        self.dimension = dimension
        self.prognostic = prognostic
        size, domainindices = variable_shape(self.param)
        self.shape = [param["nz"], param["ny"], param["nx"]]
        nzl, nyl, nxl = size
        self.size = {"i": nxl, "j": nyl, "k": nzl}
        self.domainindices = domainindices
        # index span of a multigrid-sized array (core/variables.py:114-134)
        k0, k1, j0, j1, i0, i1 = domainindices
        self.mg_idx = (slice(max(0, k0 - 1), min(nzl, k1 + 1)), slice(max(0, j0 - 1), min(nyl, j1 + 1)),
                       slice(max(0, i0 - 1), min(nxl, i1 + 1)))
        if data is None:
            data = torch.zeros((nzl, nyl, nxl), dtype=dtype, device=device)
        assert tuple(data.shape) == (nzl, nyl, nxl)
        self.data = data
        self.activeview = "i"

    def duplicate(self):
        return Scalar(self.param, self.name, self.nickname, self.dimension, self.prognostic,
                      dtype=self.data.dtype, device=self.data.device)

    def view(self, idx=None):
        """Tensor with direction `idx` innermost (core/variables.py:162-182)."""
        if idx is None:
            idx = self.activeview
        if idx not in _PERM:
            raise ValueError("argument idx of Scalar.view must be in ['i','j','k'], not " + repr(idx))
        self.activeview = idx
        return self.data.permute(*_PERM[idx])

    def flipview(self, idx):
        """Tensor with direction `idx` outermost (core/variables.py:184-204)."""
        if idx not in _FLIP:
            raise ValueError('argument idx of Scalar.flipview must be in ["i","j","k"], not ' + repr(idx))
        return self.view(_FLIP[idx])

    def viewlike(self, scalar):
        return self.view(scalar.activeview)

    @staticmethod
    def get_nature():
        return "scalar"

    def data_ptr(self):
        return self.data.data_ptr()


class Vector(dict):
    """Three Scalars 'i', 'j', 'k' (core/variables.py:209-279)."""

    def __init__(self, param, name, nickname, dimension, prognostic=False, is_velocity=True, data=None,
                 dtype=torch.float64, device="cpu"):
        dirname = {"i": "x", "j": "y", "k": "z"}
        for n, d in enumerate("ijk"):
            self[d] = Scalar(param, name + " %s-component" % dirname[d], nickname + "_" + d, dimension,
                             prognostic, data=None if data is None else data[n], dtype=dtype, device=device)
        self.param = self["i"].param
        self.name = name
        self.nickname = nickname
        self.dimension = dimension
        self.prognostic = prognostic
        self.is_velocity = is_velocity

    def duplicate(self):
        return Vector(self.param, self.name, self.nickname, self.dimension, self.prognostic, self.is_velocity,
                      dtype=self["i"].data.dtype, device=self["i"].data.device)

    def get_nature(self):
        return "velocity" if self.is_velocity else "vorticity"


class State(object):
    """Container of the model variables (core/variables.py:284-383)."""

    def __init__(self, listvar, storage=None):
        self.toc = {}
        self.storage = storage
        for var in listvar:
            self.toc[var.nickname] = var.get_nature()
            setattr(self, var.nickname, var)

    def __str__(self):
        return "\n".join("{:10}: {!r}".format(v, getattr(self, v)) for v in self.toc)

    def duplicate_prognostic_variables(self):
        return State([getattr(self, v).duplicate() for v in self.toc if getattr(self, v).prognostic])

    def get(self, variable):
        if len(variable) > 2 and variable[-2] == "_" and variable[-1] in "ijk":
            return getattr(self, variable[:-2])[variable[-1]]
        return getattr(self, variable)

    def get_prognostic_variables(self):
        return [v for v in self.toc if getattr(self, v).prognostic]

    def get_prognostic_scalars(self):
        out = []
        for nickname in self.get_prognostic_variables():
            if self.toc[nickname] == "scalar":
                out.append(nickname)
            else:
                out += ["{}_{}".format(nickname, d) for d in "ijk"]
        return out

    def scalars(self):
        """Every Scalar in field-id order: b p ke div u_i u_j u_k U_i U_j U_k vor_i vor_j vor_k work t0.."""
        out = []
        for name, nature in self.toc.items():
            if nature == "scalar":
                out.append(getattr(self, name))
            else:
                out += [getattr(self, name)[d] for d in "ijk"]
        return out


def tracer_names(n_tracers):
    return ["t{}".format(i) for i in range(n_tracers)]


def get_state(param, dtype=torch.float64, device="cpu", arena=None):
    """Full model state in one (nfields, nz, ny, nx) tensor; tracers t0.. come last
    (core/model_les.py:36-44, core/variables.py:414-437). With `arena` (an Arena) the
    tensor is carved from its buffer instead of allocated."""
    ntr = param.get("n_tracers", 0)
    size, _ = variable_shape(param)
    nf = 14 + ntr
    if arena is not None:
        storage = arena.take((nf,) + tuple(size), dtype)
    else:
        storage = torch.zeros((nf,) + tuple(size), dtype=dtype, device=device)
    listvar, k = [], 0
    for nickname, var in modelvar.items():
        if var.type == "scalar":
            listvar.append(Scalar(param, var.name, nickname, var.dimension, var.prognostic, data=storage[k]))
            k += 1
        else:
            listvar.append(Vector(param, var.name, nickname, var.dimension, var.prognostic,
                                  is_velocity=(var.type == "velocity"), data=storage[k:k + 3]))
            k += 3
    for i, t in enumerate(tracer_names(ntr)):
        listvar.append(Scalar(param, "tracer{}".format(i), t, "", True, data=storage[k]))
        k += 1
    return State(listvar, storage=storage)


def get_prognostic_registers(param, nreg, dtype=torch.float64, device="cpu", arena=None):
    """`nreg` States of the prognostic variables (b, u, t0..) in one tensor
    (nreg, nprog, nz, ny, nx) — the time-scheme registers (core/timescheme.py:92-101)."""
    ntr = param.get("n_tracers", 0)
    size, _ = variable_shape(param)
    nprog = 4 + ntr
    if arena is not None:
        storage = arena.take((nreg, nprog) + tuple(size), dtype)
    else:
        storage = torch.zeros((nreg, nprog) + tuple(size), dtype=dtype, device=device)
    states = []
    for r in range(nreg):
        lv = [Scalar(param, "buoyancy", "b", "L.T^-2", True, data=storage[r, 0]),
              Vector(param, "covariant velocity", "u", "L^2.T^-1", True, True, data=storage[r, 1:4])]
        for i, t in enumerate(tracer_names(ntr)):
            lv.append(Scalar(param, "tracer{}".format(i), t, "", True, data=storage[r, 4 + i]))
        states.append(State(lv, storage=storage[r]))
    return states, storage


class Arena(object):
    """Sub-allocations from one uint8 device buffer, each 256-byte aligned, handed out in
    call order. Models built in arenas of the same size from the same parameters get the
    same layout (each array at the same offset), which batched launches rely on: one
    run's memory is another's shifted by the distance between their buffers. The buffer
    must start zeroed, as fresh allocations are."""

    ALIGN = 256

    def __init__(self, buf):
        if buf.dtype != torch.uint8 or buf.dim() != 1:
            raise ValueError("an Arena takes a 1-D uint8 tensor")
        self.buf = buf
        self.used = 0

    @staticmethod
    def aligned(nbytes):
        return (int(nbytes) + Arena.ALIGN - 1) // Arena.ALIGN * Arena.ALIGN

    def take(self, shape, dtype):
        esize = torch.empty(0, dtype=dtype).element_size()
        n = esize
        for d in shape:
            n *= int(d)
        start = self.aligned(self.buf.data_ptr() + self.used) - self.buf.data_ptr()
        if start + n > self.buf.numel():
            raise MemoryError("arena of %d bytes exhausted (%d more needed)" % (self.buf.numel(), start + n))
        self.used = start + n
        return self.buf[start:start + n].view(dtype).view(tuple(shape))
