"""Vortex-force work diagnostic (core/online_diag.py:11-35) on the CPU: the oracle's
restatement against the reference's own VFwork run on the golden final states, and the
summed box of the reference's slice of its (j, i, k)-ordered array."""
import types

import numpy as np
import pytest

import helpers
import oracle
from nyles_gb300 import online_diag


def grid_like(meta):
    nx, ny, nz = meta["n"]
    g = meta["geometry"]
    hx, hy, hz = (3 if "x" in g else 0), (3 if "y" in g else 0), (3 if "z" in g else 0)
    return types.SimpleNamespace(domainindices=(hz, hz + nz, hy, hy + ny, hx, hx + nx),
                                 size={"i": nx + 2 * hx, "j": ny + 2 * hy, "k": nz + 2 * hz})


def test_reference_box_is_the_interior_of_a_cube():
    g = types.SimpleNamespace(domainindices=(3, 11, 3, 11, 3, 11), size={"i": 14, "j": 14, "k": 14})
    assert online_diag.reference_box(g) == online_diag.interior_box(g)


def test_reference_box_of_a_perio_xy_box():
    # arrays (8, 14, 14): the slice [0:8, 3:11, 3:11] of the (j, i, k) array covers
    # y in 0:8, x in 3:11, z in 3:8
    g = types.SimpleNamespace(domainindices=(0, 8, 3, 11, 3, 11), size={"i": 14, "j": 14, "k": 8})
    assert online_diag.reference_box(g) == (3, 8, 0, 8, 3, 11)


@pytest.mark.parametrize("name", helpers.golden_cases())
def test_oracle_vfwork_matches_reference(name):
    d, meta = helpers.load_golden(name)
    nx, ny, nz = meta["n"]
    visc = (meta.get("diff_coef") or {}).get("u")
    o = oracle.OracleModel(dict(nx=nx, ny=ny, nz=nz, nh=3, geometry=meta["geometry"], n_tracers=meta["n_tracers"],
                                modelname=meta["modelname"], timestepping=meta["timestepping"], dx=meta["dx"],
                                dy=meta["dy"], dz=meta["dz"], idx2=meta["idx2"], idy2=meta["idy2"],
                                idz2=meta["idz2"], fparam=meta["fparam"], visc=visc))
    progs = helpers.PROG + ["t%d" % i for i in range(meta["n_tracers"])]
    for s in progs + helpers.DIAG:
        o.field(s)[...] = d["final_" + s]
    total = o.vfwork(online_diag.reference_box(grid_like(meta)))
    for q, c in enumerate("ijk"):
        np.testing.assert_array_equal(o.register(0, 1 + q), d["vfwork_du_" + c], err_msg=c)
    np.testing.assert_array_equal(o.field("work"), d["vfwork_work"])
    scale = np.abs(d["vfwork_work"]).sum()
    assert abs(total - float(d["vfwork_sum"])) <= 1e-13 * scale
