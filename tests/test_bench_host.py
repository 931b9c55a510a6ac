"""Host arithmetic of bench.py on the CPU: the multigrid level model, the one-block
coarse-level rule it mirrors, the roofline fractions and the whole-job value. bench.py
is imported inside each test (it sets a CUDA environment variable when imported)."""
import os
import sys

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def _bench():
    sys.path.insert(0, os.path.dirname(HERE))
    import bench
    return bench


def test_levels_and_coarse_rule():
    b = _bench()
    lev = b.mg_levels(256)
    assert lev[0] == (256, 256, 256) and lev[-1] == (2, 2, 2) and len(lev) == 8
    # FP32: 16^3 and below fit in 200 KB (3 arrays); FP64: capped at 1024 cells (8^3)
    assert lev[b.mg_bottom_level(lev, 4)] == (16, 16, 16)
    assert lev[b.mg_bottom_level(lev, 8)] == (8, 8, 8)
    # never level 0, two levels at least
    small = b.mg_levels(4)
    assert b.mg_bottom_level(small, 4) >= 1


def test_roofline_fractions_follow_the_phase_times():
    b = _bench()
    ph = {"rhs": {"count": 3, "ms": 3.0}, "mg_norm": {"count": 10, "ms": 9.0}}
    r = b.roofline("rhs", ph, 256, 4, 6778.0, "measured", None)
    assert r["bytes_per_launch"] == 12 * 4 * 256 ** 3
    assert r["achieved"] == pytest.approx(12 * 4 * 256 ** 3 / 1e-3 / 1e9)
    assert r["frac"] == pytest.approx(r["achieved"] / 6778.0)
    n1 = b.roofline("mg_norm", ph, 256, 4, 6778.0, "measured", None, nv=10.0, solves=3, krylov=True)
    n2 = b.roofline("mg_norm", ph, 256, 4, 6778.0, "measured", None, nv=10.0, solves=6, krylov=True)
    assert n2["frac"] == pytest.approx(2 * n1["frac"])
    assert b.roofline("mg_smooth", ph, 256, 4, 6778.0, "measured", None) is None   # no such phase
    # FP64 smoothing: 5 grid levels above the one-block 8^3 bottom, one bracketed call
    # per smoothing and the coarse solve (2 x 5 + 1 per V-cycle)
    sm = b.roofline("mg_smooth", {"mg_smooth": {"count": 11 * 4, "ms": 8.0}}, 256, 8, 6778.0, "measured", None)
    assert sm["vcycles"] == pytest.approx(4.0)
    assert sm["frac"] == pytest.approx(sm["bytes_per_vcycle"] * 4 / 8e-3 / 1e9 / 6778.0)


def test_step_bytes_and_job_value():
    b = _bench()
    assert b.step_bytes("mixed", 4, 11, krylov=True) > b.step_bytes("mixed", 4, 10, krylov=True)
    assert b.step_bytes("fp64", 4, 17) > b.step_bytes("mixed", 4, 17, refine=False)
    assert b.job_value(256 ** 3, 5, 1000.0, 2) == pytest.approx(2 * 256 ** 3 * 5)
