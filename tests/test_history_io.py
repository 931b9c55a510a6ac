"""History files (core/nylesIO.py) on the CPU: file layout, names, units, parameter
attributes, frames appended at history times, variable selection and errors; the
classic-format writer against scipy's independent reader."""
import os

import numpy as np
import pytest
from scipy.io import netcdf_file

from nyles_gb300 import grid as grid_module
from nyles_gb300 import ncwriter
from nyles_gb300 import nylesIO
from nyles_gb300 import parameters
from nyles_gb300 import topology as topo
from nyles_gb300 import variables as var


def _setup(tmp_path, geometry="perio_xy", n=(8, 6, 4), **io):
    parameters.InextensibleDict.unfreeze()
    up = parameters.UserParameters()
    param = dict(up.view_parameters())
    nx, ny, nz = n
    param.update(nx=nx, ny=ny, nz=nz, npx=1, npy=1, npz=1, Lx=2.0, Ly=1.5, Lz=1.0, loc=[0, 0, 0], myrank=0,
                 geometry=geometry, neighbours=topo.get_neighbours([0, 0, 0], [1, 1, 1], geometry),
                 datadir=str(tmp_path), expname="exp", timestep_history=0.5)
    param.update(io)
    g = grid_module.Grid(param)
    st = var.get_state(param)
    rng = np.random.default_rng(0)
    for s in st.scalars():
        s.data.copy_(__import__("torch").from_numpy(rng.standard_normal(tuple(s.data.shape))))
    return param, g, st


def test_layout_and_frames(tmp_path):
    param, g, st = _setup(tmp_path)
    io = nylesIO.NylesIO(param)
    assert io.hist_path == str(tmp_path / "exp" / "exp_00_hist.nc")
    io.init(st, g, 0.0, 0)
    b0 = st.b.view("i").numpy().copy()
    st.b.view("i").add_(1.0)
    assert io.write(st, 0.25, 1) is False          # before the next history time: nothing
    io.write(st, 0.5, 2)
    io.flush()
    k0, k1, j0, j1, i0, i1 = g.domainindices
    dims, gatts, v = ncwriter.read(io.hist_path)
    dims = dict(dims)
    assert dims["t"] == 0                            # the unlimited dimension
    assert dims["x_b"] == 8 and dims["y_vor_k"] == 6 and dims["z_w"] == 4
    assert set(v) >= {"n", "t", "b", "u", "v", "w", "x_b", "y_v", "z_vor_i"}
    assert list(v["t"][1]) == [0.0, 0.5] and list(v["n"][1]) == [0, 2]
    np.testing.assert_array_equal(v["b"][1][0], b0[k0:k1, j0:j1, i0:i1])
    np.testing.assert_array_equal(v["b"][1][1], b0[k0:k1, j0:j1, i0:i1] + 1.0)
    np.testing.assert_array_equal(v["x_u"][1], g.x_u_1D[i0:i1])
    assert v["u"][1].shape == (2, 4, 6, 8)
    assert v["v"][0]["long_name"] == "covariant velocity y-component"
    assert v["t"][0]["units"] == "s"
    assert v["x_v"][0]["long_name"] == "x at cell faces y-component"
    assert gatts["geometry"] == "perio_xy" and gatts["nx"] == 8
    assert gatts["rotating"] == "False" and gatts["mode"] == "overwrite"


def test_simplified_grid_halo_and_selection(tmp_path):
    param, g, st = _setup(tmp_path, simplified_grid=True, include_halo=True, variables_in_history="p+p",
                          n_tracers=0)
    io = nylesIO.NylesIO(param)
    io.init(st, g)
    io.close()
    dims, _, v = ncwriter.read(io.hist_path)
    dims = dict(dims)
    assert dims["x"] == 8 + 6 and dims["z"] == 4
    assert {"b", "u", "v", "w", "p", "x", "y", "z"} <= set(v)
    assert v["p"][1].shape == (1, 4, 6 + 6, 8 + 6)
    np.testing.assert_array_equal(v["p"][1][0], st.p.view("i").numpy())


def test_classic_writer_against_scipy(tmp_path):
    """A file of the writer read back by scipy's netCDF reader (attribute names it can
    hold): dimensions, types, attributes, fixed data and records; each append grows the
    file by one record."""
    path = str(tmp_path / "a.nc")
    rng = np.random.default_rng(1)
    x = rng.standard_normal(5)
    w = ncwriter.ClassicWriter(path, [("t", None), ("z", 3), ("x", 5)], {"title": "abc", "nx": 5, "dt": 0.25},
                               [("n", ("t",), "i4", {}), ("x", ("x",), "f8", {"units": "m"}),
                                ("f", ("t", "z", "x"), "f8", {"long_name": "field"})], {"x": x})
    frames = [rng.standard_normal((3, 5)) for _ in range(3)]
    size = os.path.getsize(path)
    for k, fr in enumerate(frames):
        w.append({"n": 10 * k, "f": fr})
        assert os.path.getsize(path) == size + (k + 1) * w.recsize
    with netcdf_file(path, "r", mmap=False) as f:
        assert f.version_byte == 2
        assert f.dimensions == {"t": None, "z": 3, "x": 5}
        assert f.title == b"abc" and f.nx == 5 and f.dt == 0.25
        assert f.variables["f"].dimensions == ("t", "z", "x") and f.variables["f"].long_name == b"field"
        np.testing.assert_array_equal(f.variables["x"][:], x)
        np.testing.assert_array_equal(f.variables["n"][:], [0, 10, 20])
        np.testing.assert_array_equal(f.variables["f"][:], np.stack(frames))


def test_selection_errors_and_modes(tmp_path):
    param, g, st = _setup(tmp_path, variables_in_history=["b", "nope"])
    with pytest.raises(ValueError):
        nylesIO.NylesIO(param).init(st, g)
    param, g, st = _setup(tmp_path, variables_in_history=[])
    with pytest.raises(ValueError):
        nylesIO.NylesIO(param).init(st, g)
    param, g, st = _setup(tmp_path, mode="count")
    a = nylesIO.NylesIO(param)
    b = nylesIO.NylesIO(param)
    assert a.output_directory != b.output_directory and a.output_directory.endswith("exp_0000")
    param, g, st = _setup(tmp_path, mode="continue", expname="missing")
    with pytest.raises(ValueError):
        nylesIO.NylesIO(param)


def test_finalize_and_save_array(tmp_path):
    param, g, st = _setup(tmp_path, simplified_grid=True)
    io = nylesIO.NylesIO(param)
    io.init(st, g, 0.0, 0)
    io.write(st, 0.5, 3)
    io.finalize(st, 0.5, 3)                          # step 3 is already the last frame
    io.finalize(st, 0.7, 4)
    extra = np.arange(4 * 6 * 8, dtype=np.float64).reshape(4, 6, 8)
    io.save_array_3D(extra, "extra", "an added field")
    with pytest.raises(ValueError):
        io.save_array_3D(extra, "extra")
    dims, gatts, v = ncwriter.read(io.hist_path)
    assert list(v["n"][1]) == [0, 3, 4] and list(v["t"][1]) == [0.0, 0.5, 0.7]
    np.testing.assert_array_equal(v["extra"][1], extra)
    assert v["extra"][0]["long_name"] == "an added field"
    k0, k1, j0, j1, i0, i1 = g.domainindices
    np.testing.assert_array_equal(v["b"][1][2], st.b.view("i").numpy()[k0:k1, j0:j1, i0:i1])
    # frames appended after the rewrite land behind the old ones
    io.write(st, 1.0, 5)
    io.flush()
    assert list(ncwriter.read(io.hist_path)[2]["n"][1]) == [0, 3, 4, 5]
