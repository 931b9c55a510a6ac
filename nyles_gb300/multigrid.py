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
        """Device tensor aliasing a level array (var 1 = x, 2 = b): float64 (fp64) or
        float32 (mixed); level 1 of the mixed solver holds float pairs (hi, lo), shape
        (nz, ny, nx, 2), whose value is hi + lo."""
        p = ctypes.c_void_p()
        nat.check(self.lib.nyles_mg_level_ptr(self._h, lev, var, ctypes.byref(p)))
        shape = self.level_shape(lev)
        n = shape[0] * shape[1] * shape[2]
        if self.precision == "fp64":
            return _alias(self.workspace, p.value - self.workspace.data_ptr(), n, torch.float64).view(shape)
        if lev == 1:
            return _alias(self.workspace, p.value - self.workspace.data_ptr(), 2 * n, torch.float32).view(shape + (2,))
        return _alias(self.workspace, p.value - self.workspace.data_ptr(), n, torch.float32).view(shape)

    def get(self, lev, var):
        """float64 copy of a level array (pairs summed)."""
        t = self.level_tensor(lev, var)
        if self.precision != "fp64" and lev == 1:
            return t[..., 0].double() + t[..., 1].double()
        return t.double()

    def set(self, lev, var, value):
        """write a level array from any float tensor (split into pairs where needed)"""
        t = self.level_tensor(lev, var)
        v = torch.as_tensor(value, device=self.device).reshape(self.level_shape(lev)).double()
        if self.precision != "fp64" and lev == 1:
            hi = v.float()
            t[..., 0].copy_(hi)
            t[..., 1].copy_((v - hi.double()).float())
        else:
            t.copy_(v)

    def set_params(self, tol=1e-6, maxite=20, omega=0.9):
        nat.check(self.lib.nyles_mg_set_params(self._h, float(tol), int(maxite), float(omega)))

    def set_krylov(self, on=True):
        """Mixed precision: FCG(1) preconditioned by the FP32 V-cycle instead of the
        stationary V-cycle iteration (same stop rule)."""
        nat.check(self.lib.nyles_mg_set_krylov(self._h, 1 if on else 0))

    def solve(self, b=None):
        """Solve with the current warm start; `b` (interior, any dtype) replaces the
        right-hand side when given. Returns (x, stats dict): x aliases the solution in
        fp64 and is a float64 copy in mixed precision."""
        if b is not None:
            self.set(1, 2, b)
        st = nat.NylesMgStats()
        rc = self.lib.nyles_mg_solve(self._h, ctypes.byref(st), nat.stream_ptr())
        if rc not in (nat.NYLES_OK, nat.NYLES_NOT_CONVERGED):
            nat.check(rc)
        x = self.level_tensor(1, 1) if self.precision == "fp64" else self.get(1, 1)
        return x, {"nite": st.nite, "res": st.res, "converged": rc == nat.NYLES_OK}


def _alias(buf, byte_offset, n, dtype):
    """float64 tensor of n elements at byte_offset inside the uint8 tensor buf."""
    esize = torch.empty(0, dtype=dtype).element_size()
    return buf[byte_offset:byte_offset + n * esize].view(dtype)
