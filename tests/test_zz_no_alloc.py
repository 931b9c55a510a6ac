"""The allocation-free CFL reduction against the workspace-based one.

nyles_max_U2_static_f64 exists for callers that cannot allocate device memory — a host
framework that owns every device allocation through a pre-sized pool, a time loop that
must not allocate between steps, or a plain C/ctypes caller without an allocator. It
keeps its block partials in a static device array instead of a workspace. Here both
entry points are called through the C ABI on the same fields, twice in a row with
different data, and must agree to the tolerance of the other kernel tests.

The grid holds more than 2^18 stored cells, so the reduction runs several blocks and the
final pass combines several partials. The first call has the larger values: a second
call that read a partial left over from the first would return the first call's
maximum. Flat arrays of 3 * 2^18 + 5 cells (four blocks) are checked against torch's
maximum, and a NaN in one component must come back as NaN.
"""
import ctypes

import numpy as np
import pytest

import helpers

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

TOL = 1e-13


def _call_static(nat, U, V, W, out, n=None):
    return nat.lib().nyles_max_U2_static_f64(ctypes.c_void_p(U.data_ptr()), ctypes.c_void_p(V.data_ptr()),
                                             ctypes.c_void_p(W.data_ptr()), U.numel() if n is None else n,
                                             ctypes.c_void_p(out.data_ptr()), nat.stream_ptr())


def test_static_scratch_reduction_matches_workspace_reduction():
    from nyles_gb300 import _native as nat
    from nyles_gb300.nyles import Nyles
    nyl = Nyles(helpers.make_params(geometry="perio_xy", n=(64, 64, 96)))
    m = nyl.model
    st = m.state
    U, V, W = st.U["i"].data, st.U["j"].data, st.U["k"].data
    assert U.numel() > 1 << 18                    # several blocks, several partials
    out = torch.full((1,), -1.0, dtype=torch.float64, device=U.device)
    rng = np.random.Generator(np.random.PCG64(11))
    for call in range(2):   # two calls in a row, the larger values first
        scale = 10.0 ** (1 - call)
        for t in (U, V, W):
            t.copy_(torch.from_numpy(scale * rng.standard_normal(tuple(t.shape))))
        expected = m.max_U2()                      # existing entry point (model workspace)
        nat.check(_call_static(nat, U, V, W, out))
        torch.cuda.synchronize()
        got = float(out.item())
        assert abs(got - expected) <= TOL * abs(expected), (call, got, expected)
    # sizes beyond the static scratch are refused before any launch
    rc = _call_static(nat, U, V, W, out, n=(1 << 28) + 1)
    assert rc == nat.NYLES_BAD_ARG
    assert b"exceed" in nat.lib().nyles_last_error()


def test_static_scratch_reduction_four_blocks_and_nan():
    from nyles_gb300 import _native as nat
    n = 3 * (1 << 18) + 5
    dev = torch.device("cuda", torch.cuda.current_device())
    g = torch.Generator(device="cpu").manual_seed(12)
    out = torch.full((1,), -1.0, dtype=torch.float64, device=dev)
    for call, scale in enumerate((4.0, 1.0)):
        U, V, W = (scale * torch.randn(n, dtype=torch.float64, generator=g)).to(dev), \
            (scale * torch.randn(n, dtype=torch.float64, generator=g)).to(dev), \
            (scale * torch.randn(n, dtype=torch.float64, generator=g)).to(dev)
        # second call: the maximum (64 + ...) sits in the last cell of the last block,
        # below the first call's maximum (about 16 * 35)
        if call == 1:
            U[-1] = 8.0
        nat.check(_call_static(nat, U, V, W, out))
        torch.cuda.synchronize()
        expected = float((U * U + V * V + W * W).max())
        got = float(out.item())
        assert abs(got - expected) <= TOL * abs(expected), (call, got, expected)
    W[n // 2] = float("nan")
    nat.check(_call_static(nat, U, V, W, out))
    torch.cuda.synchronize()
    assert np.isnan(float(out.item()))
