"""Vortex-force work diagnostic on the GPU against the reference's own VFwork output
(golden final states) and against the oracle on seeded states, FP64 and mixed."""
import numpy as np
import pytest

import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", helpers.golden_cases())
def test_vfwork_on_golden_states(name):
    from test_gpu_model import _gpu_from_golden
    nyl, d, meta = _gpu_from_golden(name)
    m = nyl.model
    progs = helpers.PROG + ["t%d" % i for i in range(meta["n_tracers"])]
    for s in progs + helpers.DIAG:
        m.state.get(s).view("i")[...] = torch.from_numpy(d["final_" + s])
    total = nyl.diag.compute()
    work = m.state.get("work").view("i").cpu().numpy()
    ref = d["vfwork_work"]
    scale = max(np.abs(ref).max(), 1e-300)
    assert np.abs(work - ref).max() <= 1e-12 * scale
    du = [m.timescheme.dstate.get("u_" + c).view("i").cpu().numpy() for c in "ijk"]
    duref = [d["vfwork_du_" + c] for c in "ijk"]
    dscale = max(max(np.abs(a).max() for a in duref), 1e-300)
    for a, b in zip(du, duref):
        assert np.abs(a - b).max() <= 1e-12 * dscale
    assert abs(total - float(d["vfwork_sum"])) <= 1e-12 * max(np.abs(ref).sum(), 1e-300)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
@pytest.mark.parametrize("cfg,kind", [
    (dict(geometry="perio_xy", n=(32, 16, 24), L=(2.0, 1.0, 1.5), n_tracers=1), "noise"),
    (dict(geometry="closed", n=(24, 24, 24)), "noise"),
    (dict(geometry="perio_xyz", n=(16, 16, 16), L=(6.283185307179586,) * 3), "tgv"),
])
def test_vfwork_against_oracle(cfg, kind, precision, tol):
    from nyles_gb300 import online_diag
    from nyles_gb300.nyles import Nyles
    nyl = Nyles(helpers.make_params(precision=precision, **cfg))
    o = helpers.oracle_for(nyl)
    helpers.load_state(nyl, o, helpers.seeded_state(nyl, kind, 7))
    nyl.model.diagnose_var(nyl.model.state)
    o.diagnose()
    for interior in (False, True):
        box = online_diag.interior_box(nyl.grid) if interior else online_diag.reference_box(nyl.grid)
        ref = o.vfwork(box)
        got = nyl.diag.compute(interior=interior)
        w_ref = o.field("work")
        w = nyl.model.state.get("work").view("i").double().cpu().numpy()
        assert np.abs(w - w_ref).max() <= tol * np.abs(w_ref).max()
        assert abs(got - ref) <= tol * np.abs(w_ref).sum()
