"""The vortex-force binding that the integration guide at the repository root (its
section 3.1) gives a reference maintainer to paste into core/vortex_force.py, executed
as written: its NylesDesc filled field by field from the package's descriptor, its
vortex_force() called on a small state, and the tendencies compared with the oracle
(the FP64 kernel bar, 1e-13)."""
import os
import re

import numpy as np
import pytest

import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _snippet():
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    return re.search(r"### 3\.1.*?```python\n(.*?)```", text, flags=re.S).group(1)


@pytest.mark.parametrize("vf", [("weno", 5), ("linear", 3)])
def test_integration_snippet_vortex_force(monkeypatch, vf):
    from nyles_gb300.nyles import Nyles
    monkeypatch.chdir(REPO)                 # the snippet opens the library by its in-tree path
    ns = {}
    exec(_snippet(), ns)
    nyl = Nyles(helpers.make_params(geometry="perio_xy", n=(16, 8, 12), n_tracers=1, vf_scheme=vf[0],
                                    orderVF=vf[1]))
    o = helpers.oracle_for(nyl)
    helpers.load_state(nyl, o, helpers.seeded_state(nyl, "noise", 31))
    rng = np.random.Generator(np.random.PCG64(32))
    st = nyl.model.state
    shape = tuple(st.b.view("i").shape)
    for name in ("U_i", "U_j", "U_k", "vor_i", "vor_j", "vor_k"):
        a = rng.standard_normal(shape)
        st.get(name).view("i")[...] = torch.from_numpy(a)
        o.field(name)[...] = a
    desc = ns["NylesDesc"]()
    src = nyl.model.desc
    for name, _ in ns["NylesDesc"]._fields_:
        v = getattr(src, name)
        if hasattr(v, "__len__"):
            for i in range(len(v)):
                getattr(desc, name)[i] = v[i]
        else:
            setattr(desc, name, v)
    ds = nyl.model.timescheme.registers[0]
    ds.storage.zero_()
    ns["vortex_force"](list(st.scalars()), list(ds.scalars()), desc)
    torch.cuda.synchronize()
    o.vortex_force(0)
    for q, name in enumerate(["u_i", "u_j", "u_k"]):
        assert helpers.relerr(ds.get(name).view("i").cpu().numpy(), o.register(0, 1 + q)) < 1e-13, name
