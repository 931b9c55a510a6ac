"""Stand-alone multigrid Poisson solver (the mgfor interface of core/mgfordriver.py).

``MG(nx, ny, nz, topology, precision)`` holds the level hierarchy in one device
workspace. ``solve(b)`` takes the interior right-hand side (nz, ny, nx) and returns
the interior solution; the level-1 solution persists between solves (warm start,
core/mgfordriver.py:66-78). Stop rule of core/mgfor/solvers.f90:8-33.
"""
import ctypes

import torch

from . import _native as nat


class MG(object):
    def __init__(self, nx, ny, nz, topology="closed", precision="fp64", device=None):
        self.lib = nat.lib()
        topo = nat.MG_TOPOLOGY[topology] if isinstance(topology, str) else int(topology)
        h = ctypes.c_void_p()
        nat.check(self.lib.nyles_mg_create(nx, ny, nz, topo, nat.PRECISION[precision], ctypes.byref(h)))
        self._h = h
        nb = ctypes.c_size_t()
        nat.check(self.lib.nyles_mg_workspace_bytes(h, ctypes.byref(nb)))
        dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.workspace = torch.zeros(nb.value + 256, dtype=torch.uint8, device=dev)
        ws = (self.workspace.data_ptr() + 255) & ~255
        nat.check(self.lib.nyles_mg_bind(h, ctypes.c_void_p(ws)))
        n = ctypes.c_int()
        nat.check(self.lib.nyles_mg_nlevels(h, ctypes.byref(n)))
        self.nlevels = n.value
        self.device = dev
        self.precision = precision
        self.shape = self.level_shape(1)

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            try:
                self.lib.nyles_mg_destroy(h)
            except Exception:
                pass
            self._h = None

    def level_shape(self, lev):
        s = (ctypes.c_int * 3)()
        nat.check(self.lib.nyles_mg_level_shape(self._h, lev, s))
        return (s[0], s[1], s[2])

    def level_tensor(self, lev, var):
        """Device tensor aliasing a level array (var 1 = x, 2 = b). Level 1 is float64;
        coarser levels are float64 (fp64) or float32 (mixed)."""
        p = ctypes.c_void_p()
        nat.check(self.lib.nyles_mg_level_ptr(self._h, lev, var, ctypes.byref(p)))
        shape = self.level_shape(lev)
        n = shape[0] * shape[1] * shape[2]
        dtype = torch.float64 if (lev == 1 or self.precision == "fp64") else torch.float32
        return _alias(self.workspace, p.value - self.workspace.data_ptr(), n, dtype).view(shape)

    def set_params(self, tol=1e-6, maxite=20, omega=0.9):
        nat.check(self.lib.nyles_mg_set_params(self._h, float(tol), int(maxite), float(omega)))

    def solve(self, b=None):
        """Solve with the current warm start; `b` (interior, any dtype) replaces the
        right-hand side when given. Returns (x view, stats dict)."""
        if b is not None:
            self.level_tensor(1, 2).copy_(torch.as_tensor(b, device=self.device).reshape(self.shape))
        st = nat.NylesMgStats()
        rc = self.lib.nyles_mg_solve(self._h, ctypes.byref(st), nat.stream_ptr())
        if rc not in (nat.NYLES_OK, nat.NYLES_NOT_CONVERGED):
            nat.check(rc)
        return self.level_tensor(1, 1), {"nite": st.nite, "res": st.res, "converged": rc == nat.NYLES_OK}


def _alias(buf, byte_offset, n, dtype):
    """float64 tensor of n elements at byte_offset inside the uint8 tensor buf."""
    esize = torch.empty(0, dtype=dtype).element_size()
    return buf[byte_offset:byte_offset + n * esize].view(dtype)
