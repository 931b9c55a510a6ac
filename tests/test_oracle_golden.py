"""The CPU oracle's C++ orchestration against golden vectors produced by the
reference's own Python modules (tests/golden/make_golden.py): bit-exact."""
import numpy as np
import pytest

import helpers
import oracle


@pytest.mark.parametrize("name", helpers.golden_cases())
def test_oracle_matches_reference_orchestration(name):
    d, meta = helpers.load_golden(name)
    nx, ny, nz = meta["n"]
    visc = (meta.get("diff_coef") or {}).get("u")
    o = oracle.OracleModel(dict(nx=nx, ny=ny, nz=nz, nh=3, geometry=meta["geometry"], n_tracers=meta["n_tracers"],
                                modelname=meta["modelname"], timestepping=meta["timestepping"], dx=meta["dx"],
                                dy=meta["dy"], dz=meta["dz"], idx2=meta["idx2"], idy2=meta["idy2"],
                                idz2=meta["idz2"], fparam=meta["fparam"], visc=visc))
    progs = helpers.PROG + ["t%d" % i for i in range(meta["n_tracers"])]
    for s in progs:
        o.field(s)[...] = d["init_" + s]
    o.diagnose()
    assert o.mg_stats()[0] == int(d["nite_0"])
    t = 0.0
    for n in range(meta["steps"]):
        dt = o.compute_dt(meta["auto_dt"], meta.get("dt", 0.1), meta.get("cfl", 1.0), meta.get("dt_max", 1.0))
        assert dt == d["dts"][n]
        o.forward(t, dt)
        t += dt
        assert o.mg_stats()[0] == int(d["nites_last"][n])
    for s in progs + helpers.DIAG:
        np.testing.assert_array_equal(o.field(s), d["final_" + s], err_msg=s)
