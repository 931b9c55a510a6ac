"""Grid of one subdomain: spacings, metric terms and staggered coordinates.

Same attributes as the reference's core/grid.py:14-158. Coordinates are kept on the
host as float64 tensors (numpy-compatible), so initial states can be written with
numpy expressions; the model state itself lives on the GPU. The 3-D coordinate fields
(x_b, y_b, z_b, x_vel, ..., z_vor) are built on first access.
"""
import numpy as np
import torch

from .variables import Scalar, Vector, variable_shape

_CENTERS = ("x_b", "y_b", "z_b")
_FACES = ("x_vel", "y_vel", "z_vel")
_EDGES = ("x_vor", "y_vor", "z_vor")


class Grid(object):
    def __init__(self, param):
        self._param = param
        self.nx, self.ny, self.nz = param["nx"], param["ny"], param["nz"]
        self.npx, self.npy, self.npz = param["npx"], param["npy"], param["npz"]
        self.Lx, self.Ly, self.Lz = param["Lx"], param["Ly"], param["Lz"]
        # core/grid.py:30-57, same Python arithmetic
        self.dx = self.Lx / (self.npx * self.nx)
        self.dy = self.Ly / (self.npy * self.ny)
        self.dz = self.Lz / (self.npz * self.nz)
        self.dx2, self.dy2, self.dz2 = self.dx ** 2, self.dy ** 2, self.dz ** 2
        self.idx, self.idy, self.idz = 1 / self.dx, 1 / self.dy, 1 / self.dz
        self.idx2, self.idy2, self.idz2 = 1 / self.dx ** 2, 1 / self.dy ** 2, 1 / self.dz ** 2
        self.vol = self.dx * self.dy * self.dz
        self.ids2 = {"i": self.idx2, "j": self.idy2, "k": self.idz2}
        self.vol_per_ds2 = {"i": self.vol / self.dx2, "j": self.vol / self.dy2, "k": self.vol / self.dz2}

        ext, dom = variable_shape(param)
        size = {"i": ext[2], "j": ext[1], "k": ext[0]}
        self.size = size
        self.domainindices = dom
        k0, k1, j0, j1, i0, i1 = self.domainindices
        loc = param.get("loc", [0, 0, 0])
        x0 = loc[2] * self.nx * self.dx
        y0 = loc[1] * self.ny * self.dy
        z0 = loc[0] * self.nz * self.dz
        self.x_b_1D = (np.arange(size["i"]) + 0.5 - i0) * self.dx + x0
        self.y_b_1D = (np.arange(size["j"]) + 0.5 - j0) * self.dy + y0
        self.z_b_1D = (np.arange(size["k"]) + 0.5 - k0) * self.dz + z0
        # velocity points (cell faces), core/grid.py:93-124
        self.x_u_1D = self.x_b_1D + self.dx / 2
        self.y_u_1D = self.y_b_1D.copy()
        self.z_u_1D = self.z_b_1D.copy()
        self.x_v_1D = self.x_b_1D.copy()
        self.y_v_1D = self.y_b_1D + self.dy / 2
        self.z_v_1D = self.z_b_1D.copy()
        self.x_w_1D = self.x_b_1D.copy()
        self.y_w_1D = self.y_b_1D.copy()
        self.z_w_1D = self.z_b_1D + self.dz / 2
        # vorticity points (cell edges), core/grid.py:126-158
        self.x_vor_i_1D = self.x_b_1D.copy()
        self.y_vor_i_1D = self.y_b_1D + self.dy / 2
        self.z_vor_i_1D = self.z_b_1D + self.dz / 2
        self.x_vor_j_1D = self.x_b_1D + self.dx / 2
        self.y_vor_j_1D = self.y_b_1D.copy()
        self.z_vor_j_1D = self.z_b_1D + self.dz / 2
        self.x_vor_k_1D = self.x_b_1D + self.dx / 2
        self.y_vor_k_1D = self.y_b_1D + self.dy / 2
        self.z_vor_k_1D = self.z_b_1D.copy()

    @staticmethod
    def _fill(sx, sy, sz, x1, y1, z1):
        Z, Y, X = np.meshgrid(z1, y1, x1, indexing="ij")
        sz.view("i")[...] = torch.from_numpy(Z)
        sy.view("i")[...] = torch.from_numpy(Y)
        sx.view("i")[...] = torch.from_numpy(X)

    def __getattr__(self, name):
        # build the 3-D coordinate fields of a point family on first use
        prm = self.__dict__.get("_param")
        if prm is None:
            raise AttributeError(name)
        if name in _CENTERS:
            s = [Scalar(prm, "%s at cell centers" % a, "%s_b" % a, "L") for a in "xyz"]
            self._fill(*s, self.x_b_1D, self.y_b_1D, self.z_b_1D)
            self.x_b, self.y_b, self.z_b = s
        elif name in _FACES:
            v = [Vector(prm, "%s at cell faces" % a, "%s_vel" % a, "L", is_velocity=True) for a in "xyz"]
            self._fill(v[0]["i"], v[1]["i"], v[2]["i"], self.x_u_1D, self.y_u_1D, self.z_u_1D)
            self._fill(v[0]["j"], v[1]["j"], v[2]["j"], self.x_v_1D, self.y_v_1D, self.z_v_1D)
            self._fill(v[0]["k"], v[1]["k"], v[2]["k"], self.x_w_1D, self.y_w_1D, self.z_w_1D)
            self.x_vel, self.y_vel, self.z_vel = v
        elif name in _EDGES:
            v = [Vector(prm, "%s at cell edges" % a, "%s_vor" % a, "L", is_velocity=False) for a in "xyz"]
            self._fill(v[0]["i"], v[1]["i"], v[2]["i"], self.x_vor_i_1D, self.y_vor_i_1D, self.z_vor_i_1D)
            self._fill(v[0]["j"], v[1]["j"], v[2]["j"], self.x_vor_j_1D, self.y_vor_j_1D, self.z_vor_j_1D)
            self._fill(v[0]["k"], v[1]["k"], v[2]["k"], self.x_vor_k_1D, self.y_vor_k_1D, self.z_vor_k_1D)
            self.x_vor, self.y_vor, self.z_vor = v
        else:
            raise AttributeError(name)
        return self.__dict__[name]
