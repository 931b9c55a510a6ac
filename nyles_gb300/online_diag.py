"""Online diagnostic: pointwise work of the vortex force (core/online_diag.py:4-35).

``VFwork(model, grid).compute()`` recomputes the vortex force into the u components of
the time scheme's first register (as the reference does, which overwrites them), fills
``state.work`` with sum_d (U_d F_d / 2)(p) + (U_d F_d / 2)(p - e_d), and sets
``worksum`` to the sum of that field, all in libnyles_gb300.so.

The reference sums ``state.work.view()[k0:k1, j0:j1, i0:i1]`` right after its last
``view('k')``, so its slices apply to an array ordered (j, i, k): the summed box is the
interior only when the three array extents and halo widths agree. ``compute()`` sums
that same box by default (the reference's printed "Kdiss"); ``interior=True`` sums the
interior cells instead.
"""
import ctypes

from . import _native as nat


def reference_box(grid):
    """(z0, z1, y0, y1, x0, x1) that the reference's slice of the (j, i, k)-ordered
    array covers, with numpy's clamping of slice bounds."""
    k0, k1, j0, j1, i0, i1 = grid.domainindices
    nz, ny, nx = grid.size["k"], grid.size["j"], grid.size["i"]

    def clamp(lo, hi, n):
        hi = min(hi, n)
        return min(lo, hi), hi

    z = clamp(i0, i1, nz)
    y = clamp(k0, k1, ny)
    x = clamp(j0, j1, nx)
    return z + y + x


def interior_box(grid):
    k0, k1, j0, j1, i0, i1 = grid.domainindices
    return (k0, k1, j0, j1, i0, i1)


class VFwork:
    """diagnose the pointwise vortex-force work"""

    def __init__(self, model, grid):
        self.model = model
        self.grid = grid
        self.worksum = 0.0

    def compute(self, interior=False):
        box = interior_box(self.grid) if interior else reference_box(self.grid)
        b = (ctypes.c_longlong * 6)(*[int(v) for v in box])
        out = ctypes.c_double()
        nat.check(self.model.lib.nyles_model_vfwork(self.model._h, b, ctypes.byref(out), nat.stream_ptr()))
        self.worksum = out.value
        return self.worksum
