"""The allocation-free CFL reduction against the workspace-based one.

nyles_max_U2_static_f64 exists for callers that cannot allocate device memory — a host
framework that owns every device allocation through a pre-sized pool, a time loop that
must not allocate between steps, or a plain C/ctypes caller without an allocator. It
keeps its block partials in a static device array instead of a workspace. Here both
entry points are called through the C ABI on the same fields, twice in a row with
different data, and must agree to the tolerance of the other kernel tests.
"""
import ctypes

import numpy as np
import pytest

import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-13


def _call_static(nat, U, V, W, out):
    return nat.lib().nyles_max_U2_static_f64(ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(V.data_ptr()),
                                             ctypes.c_void_p(W.data_ptr()), U.numel(),
                                             ctypes.c_void_p(out.data_ptr()), nat.stream_ptr())


def test_static_scratch_reduction_matches_workspace_reduction():
    from nyles_gb300 import _native as nat
    from nyles_gb300.nyles import Nyles
    nyl = Nyles(helpers.make_params(geometry="perio_xy", n=(32, 16, 16)))
    m = nyl.model
    st = m.state
    U, V, W = st.U["i"].data, st.U["j"].data, st.U["k"].data
    out = torch.full((1,), -1.0, dtype=torch.float64, device=U.device)
    rng = np.random.Generator(np.random.PCG64(11))
    for call in range(2):   # two calls in a row; the second must not see the first's partials
        scale = 10.0 ** call
        for t in (U, V, W):
            t.copy_(torch.from_numpy(scale * rng.standard_normal(tuple(t.shape))))
        expected = m.max_U2()                      # existing entry point (model workspace)
        nat.check(_call_static(nat, U, V, W, out))
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - expected) <= TOL * abs(expected), (call, got, expected)
    # sizes beyond the static scratch are refused before any launch
    rc = nat.lib().nyles_max_U2_static_f64(ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(V.data_ptr()),
                                           ctypes.c_void_p(W.data_ptr()), (1 << 28) + 1,
                                           ctypes.c_void_p(out.data_ptr()), nat.stream_ptr())
    assert rc == nat.NYLES_BAD_ARG
    assert b"exceed" in nat.lib().nyles_last_error()
