"""Host-side logic of the package on the CPU: parameters, topology, views, grid."""
import json
import os

import numpy as np
import pytest
import torch

from nyles_gb300 import parameters as P
from nyles_gb300 import topology as topo
from nyles_gb300 import variables as var
from nyles_gb300.grid import Grid

HERE = os.path.dirname(os.path.abspath(__file__))


def test_parameter_errors_match_reference():
    cases = json.load(open(os.path.join(HERE, "golden", "params_cases.json")))
    for c in cases:
        P.InextensibleDict.unfreeze()
        p = P.UserParameters()
        err = None
        try:
            if c.get("new_key"):
                p.model["foo"] = 1
            elif c["key"] == "npz>global_nz":
                p.discretization["global_nz"] = 1
                p.MPI["npz"] = 2
                p.check()
            else:
                getattr(p, c["category"])[c["key"]] = c["value"]
                p.check()
        except P.UserParameterError as e:
            err = str(e)
        assert err == c["error"], c


def test_freeze_is_global_and_defaults_check():
    p = P.UserParameters()
    p.check()
    p.freeze()
    q = P.UserParameters()
    with pytest.raises(P.UserParameterError):
        q.model["Lx"] = 2.0
    P.InextensibleDict.unfreeze()
    with pytest.raises(P.DefaultsFileError):
        P.UserParameters.check_defaults({"model": {}})
    assert "gpu" not in P.CATEGORIES and p.gpu["precision"] == "fp64"


def test_neighbours_and_shapes():
    ngb = topo.get_neighbours([0, 0, 0], [1, 1, 1], "perio_xy")
    assert len(ngb) == 8 and (0, 1, 1) in ngb and (1, 0, 0) not in ngb
    size, dom = topo.get_variable_shape([32, 32, 64], ngb, 3)
    assert size == [32, 38, 70] and dom == (0, 32, 3, 35, 3, 67)
    assert len(topo.get_neighbours([0, 0, 0], [1, 1, 1], "perio_xyz")) == 26
    assert topo.get_neighbours([0, 0, 0], [1, 1, 1], "closed") == {}


def test_neighbour_graph_symmetric_multi_rank():
    """core/mpi/topology.py:224-250 check_graph, simulated in one process."""
    procs = [2, 2, 4]
    for geo in ("closed", "perio_x", "perio_xy", "perio_xyz"):
        n = int(np.prod(procs))
        conn = np.zeros((n, n), dtype=int)
        for r in range(n):
            for k, j in topo.get_neighbours(r, procs, geo).items():
                conn[r, j] += 1
        assert (conn == conn.T).all()


def _param(geometry="perio_xy", n=(8, 6, 4)):
    ngb = topo.get_neighbours([0, 0, 0], [1, 1, 1], geometry)
    return dict(nx=n[0], ny=n[1], nz=n[2], nh=3, neighbours=ngb, npx=1, npy=1, npz=1, Lx=2.0, Ly=1.0, Lz=0.5,
                loc=[0, 0, 0])


def test_views_are_the_reference_transposes():
    prm = _param()
    st = var.get_state(prm)
    b = st.b
    a = np.random.default_rng(0).standard_normal(tuple(b.view("i").shape))
    b.view("i")[...] = torch.from_numpy(a)
    # core/variables.py:406-411: rightswap = transpose(2,0,1), leftswap = transpose(1,2,0)
    np.testing.assert_array_equal(b.view("j").numpy(), np.transpose(a, (2, 0, 1)))
    np.testing.assert_array_equal(b.view("k").numpy(), np.transpose(a, (1, 2, 0)))
    np.testing.assert_array_equal(b.flipview("k").numpy(), a)
    b.view("j")[0, 0, 0] = 7.0          # writes land in the field
    assert b.view("i")[0, 0, 0] == 7.0
    assert st.get_prognostic_scalars() == ["b", "u_i", "u_j", "u_k"]
    assert [s.nickname for s in st.scalars()][:7] == ["b", "p", "ke", "div", "u_i", "u_j", "u_k"]


def test_grid_coordinates():
    prm = _param("closed", (8, 4, 2))
    g = Grid(prm)
    assert g.dx == 0.25 and g.idx2 == 16.0
    xb = g.x_b.view("i").numpy()
    assert xb[0, 0, 0] == 0.125 and xb.shape == (2, 4, 8)
    assert g.x_vel["i"].view("i").numpy()[0, 0, -1] == 2.0     # east wall face
    assert g.z_vor["k"].view("i").numpy()[1, 0, 0] == pytest.approx(0.375)


def test_gpu_parameter_choices_cover_the_model_modes():
    """Every mg_warm_start and mg_krylov value the model understands passes the
    parameter check, and the warm start the parameters select at creation follows
    the tolerance (the Krylov solve's extrapolated start, else the reference's)."""
    from nyles_gb300 import model_les as M
    for warm in M.WARM_STARTS:
        P.InextensibleDict.unfreeze()
        p = P.UserParameters()
        p.gpu["precision"] = "mixed"
        p.gpu["mg_warm_start"] = warm
        p.check()
    for kry in ("auto", "on", "off"):
        P.InextensibleDict.unfreeze()
        p = P.UserParameters()
        p.gpu["mg_krylov"] = kry
        p.check()
    P.InextensibleDict.unfreeze()
    assert M.creation_warm_mode({"mg_tol": 1e-20}, "mixed") == M.WARM_STARTS[M.WARM_AUTO]
    assert M.creation_warm_mode({"mg_tol": 1e-6}, "mixed") == 0
    assert M.creation_warm_mode({"mg_tol": 1e-20}, "fp64") == 0
    assert M.creation_warm_mode({"mg_tol": 1e-6, "mg_warm_start": "stage"}, "mixed") == 1
    with pytest.raises(ValueError):
        M.creation_warm_mode({"mg_warm_start": "stage"}, "fp64")
