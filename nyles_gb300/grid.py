"""Grid of one subdomain: spacings, metric terms and staggered coordinates.

Same attributes as the reference's core/grid.py:14-158. Coordinates are kept on the
host as float64 tensors (numpy-compatible), so initial states can be written with
numpy expressions; the model state itself lives on the GPU.
"""
import numpy as np
import torch

from .variables import Scalar, Vector


class Grid(object):
    def __init__(self, param):
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

        self.x_b = Scalar(param, "x at cell centers", "x_b", "L")
        self.y_b = Scalar(param, "y at cell centers", "y_b", "L")
        self.z_b = Scalar(param, "z at cell centers", "z_b", "L")
        size = self.x_b.size
        self.size = size
        self.domainindices = self.x_b.domainindices
        k0, k1, j0, j1, i0, i1 = self.domainindices
        loc = param.get("loc", [0, 0, 0])
        x0 = loc[2] * self.nx * self.dx
        y0 = loc[1] * self.ny * self.dy
        z0 = loc[0] * self.nz * self.dz
        self.x_b_1D = (np.arange(size["i"]) + 0.5 - i0) * self.dx + x0
        self.y_b_1D = (np.arange(size["j"]) + 0.5 - j0) * self.dy + y0
        self.z_b_1D = (np.arange(size["k"]) + 0.5 - k0) * self.dz + z0

        def setc(sx, sy, sz, x1, y1, z1):
            Z, Y, X = np.meshgrid(z1, y1, x1, indexing="ij")
            sz.view("i")[...] = torch.from_numpy(Z)
            sy.view("i")[...] = torch.from_numpy(Y)
            sx.view("i")[...] = torch.from_numpy(X)

        setc(self.x_b, self.y_b, self.z_b, self.x_b_1D, self.y_b_1D, self.z_b_1D)

        # velocity points (cell faces), core/grid.py:93-124
        self.x_vel = Vector(param, "x at cell faces", "x_vel", "L", is_velocity=True)
        self.y_vel = Vector(param, "y at cell faces", "y_vel", "L", is_velocity=True)
        self.z_vel = Vector(param, "z at cell faces", "z_vel", "L", is_velocity=True)
        self.x_u_1D = self.x_b_1D + self.dx / 2
        self.y_u_1D = self.y_b_1D.copy()
        self.z_u_1D = self.z_b_1D.copy()
        self.x_v_1D = self.x_b_1D.copy()
        self.y_v_1D = self.y_b_1D + self.dy / 2
        self.z_v_1D = self.z_b_1D.copy()
        self.x_w_1D = self.x_b_1D.copy()
        self.y_w_1D = self.y_b_1D.copy()
        self.z_w_1D = self.z_b_1D + self.dz / 2
        setc(self.x_vel["i"], self.y_vel["i"], self.z_vel["i"], self.x_u_1D, self.y_u_1D, self.z_u_1D)
        setc(self.x_vel["j"], self.y_vel["j"], self.z_vel["j"], self.x_v_1D, self.y_v_1D, self.z_v_1D)
        setc(self.x_vel["k"], self.y_vel["k"], self.z_vel["k"], self.x_w_1D, self.y_w_1D, self.z_w_1D)

        # vorticity points (cell edges), core/grid.py:126-158
        self.x_vor = Vector(param, "x at cell edges", "x_vor", "L", is_velocity=False)
        self.y_vor = Vector(param, "y at cell edges", "y_vor", "L", is_velocity=False)
        self.z_vor = Vector(param, "z at cell edges", "z_vor", "L", is_velocity=False)
        self.x_vor_i_1D = self.x_b_1D.copy()
        self.y_vor_i_1D = self.y_b_1D + self.dy / 2
        self.z_vor_i_1D = self.z_b_1D + self.dz / 2
        self.x_vor_j_1D = self.x_b_1D + self.dx / 2
        self.y_vor_j_1D = self.y_b_1D.copy()
        self.z_vor_j_1D = self.z_b_1D + self.dz / 2
        self.x_vor_k_1D = self.x_b_1D + self.dx / 2
        self.y_vor_k_1D = self.y_b_1D + self.dy / 2
        self.z_vor_k_1D = self.z_b_1D.copy()
        setc(self.x_vor["i"], self.y_vor["i"], self.z_vor["i"], self.x_vor_i_1D, self.y_vor_i_1D, self.z_vor_i_1D)
        setc(self.x_vor["j"], self.y_vor["j"], self.z_vor["j"], self.x_vor_j_1D, self.y_vor_j_1D, self.z_vor_j_1D)
        setc(self.x_vor["k"], self.y_vor["k"], self.z_vor["k"], self.x_vor_k_1D, self.y_vor_k_1D, self.z_vor_k_1D)
