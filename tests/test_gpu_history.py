"""Nyles.run with history files on the GPU (core/nyles.py:119-225): frames at the history
times, each equal to the state at its step (the asynchronous device-to-host copy is not
overtaken by later steps), the final frame, param.pkl and stats.pkl."""
import os
import pickle

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_run_writes_history(tmp_path, precision):
    import torch
    from nyles_gb300 import ncwriter
    from nyles_gb300.nyles import Nyles
    p = helpers.make_params("closed", n=(32, 16, 16), dt=1e-3, precision=precision)
    p.gpu["history"] = True
    p.IO["datadir"] = str(tmp_path)
    p.IO["expname"] = "lock"
    p.IO["timestep_history"] = 0.0035
    p.IO["variables_in_history"] = "p+p"
    p.time["tend"] = 0.0095          # ends at step 10, between history times
    nyl = Nyles(p)
    fields = helpers.seeded_state(nyl, "lock", 3)
    for k, v in fields.items():
        nyl.model.state.get(k).view("i")[...] = torch.from_numpy(v)
    seen = {}

    def record(nyles, t, n):
        # device clones, stream-ordered: no host synchronisation between the steps
        seen[n] = {s: nyles.model.state.get(s).view("i").clone() for s in ("b", "u_i", "p")}

    t, n, blowup = nyl.run(verbose=False, callback=record)
    seen = {k: {s: a.double().cpu().numpy() for s, a in d.items()} for k, d in seen.items()}
    assert not blowup and n == 10
    _, gatts, v = ncwriter.read(nyl.IO.hist_path)
    frames = list(v["n"][1])
    assert frames == [0, 4, 7, 10]                   # t >= 0.0035, 0.007; then the final frame
    assert gatts["expname"] == "lock" and gatts["nx"] == 32
    for r, step in enumerate(frames[1:], start=1):
        np.testing.assert_array_equal(v["b"][1][r], seen[step]["b"])
        np.testing.assert_array_equal(v["u"][1][r], seen[step]["u_i"])
        np.testing.assert_array_equal(v["p"][1][r], seen[step]["p"])
    np.testing.assert_array_equal(v["b"][1][0], fields["b"].astype(np.float32 if precision == "mixed" else np.float64))
    assert abs(v["t"][1][-1] - t) < 1e-15
    out = nyl.IO.output_directory
    with open(os.path.join(out, "param.pkl"), "rb") as fid:
        assert pickle.load(fid)["timestep_history"] == 0.0035
    assert os.path.exists(os.path.join(out, "stats.pkl"))
