"""emsim_gb300_make_slices_noalloc against emsim_gb300_make_slices, through the C ABI.

The no-allocation entry point serves callers that cannot allocate device memory while
they run - a plugin inside a program that owns all device memory through its own pool,
or a loop that must not allocate after start-up.  It keeps its intermediate in one
static device buffer shared by every call, so it is checked on two calls in a row
(the second sees the first call's leftovers), and a plan too large for the buffer must
be refused before any work is queued.  This file is collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def lib():
    import torch  # noqa: F401

    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import _native
    return _native.load()


def _plan(lib, zs, ns, n1, n2, d):
    from emsim_gb300 import elem
    sf = elem.scattering_factors_half(zs, n1, n2, d, d)
    h = ctypes.c_void_p()
    st = lib.emsim_gb300_slice_plan_create(sf.ctypes.data_as(ctypes.c_void_p), len(zs), ns, n1, n2, 2.0, d, d, 1,
                                           ctypes.byref(h))
    assert st == 0, lib.emsim_gb300_last_error()
    return h


# 128 x 128 with 6 slices: power-of-two passes, every slice pair full; 96 x 80 with 5
# slices: the generic (non-power-of-two) path and a half-empty last slice pair
@pytest.mark.parametrize("ns,n1,n2", [(6, 128, 128), (5, 96, 80)])
def test_noalloc_matches_workspace_version_twice(lib, ns, n1, n2):
    import torch

    from oracle import multislice as om
    zs = [6, 7, 8, 16]
    plan = _plan(lib, zs, ns, n1, n2, 0.5)
    need = int(lib.emsim_gb300_make_slices_workspace_size(plan))
    assert 0 < need <= 32 * 1024 * 1024
    dev = torch.device("cuda", torch.cuda.current_device())
    ws = torch.empty(need, dtype=torch.uint8, device=dev)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    P = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    rng = np.random.default_rng(77)
    try:
        for call in range(2):
            hist = torch.from_numpy(rng.poisson(0.05 * (call + 1), (len(zs), ns, n1, n2)).astype(np.float32)).to(dev)
            ref = torch.empty((ns, n1, n2), dtype=torch.float32, device=dev)
            got = torch.full_like(ref, float("nan"))
            assert lib.emsim_gb300_make_slices(plan, P(hist), P(ref), P(ws), need, st) == 0, \
                lib.emsim_gb300_last_error()
            assert lib.emsim_gb300_make_slices_noalloc(plan, P(hist), P(got), st) == 0, lib.emsim_gb300_last_error()
            torch.cuda.synchronize()
            g, r = got.cpu().numpy(), ref.cpu().numpy()
            assert np.isfinite(g).all()
            assert om.rel_l2(g, r) < TOL, call
    finally:
        lib.emsim_gb300_slice_plan_destroy(plan)


def test_noalloc_rejects_plan_larger_than_buffer(lib):
    import torch
    plan = _plan(lib, [6, 7, 8, 16], 40, 512, 512, 0.5)  # needs 4 x 20 x 512^2 x 8 B = 168 MB
    try:
        assert int(lib.emsim_gb300_make_slices_workspace_size(plan)) > 32 * 1024 * 1024
        dev = torch.device("cuda", torch.cuda.current_device())
        hist = torch.zeros((4, 40, 512, 512), dtype=torch.float32, device=dev)
        out = torch.zeros((40, 512, 512), dtype=torch.float32, device=dev)
        st = lib.emsim_gb300_make_slices_noalloc(plan, ctypes.c_void_p(hist.data_ptr()),
                                                 ctypes.c_void_p(out.data_ptr()), None)
        assert st == 3  # EMSIM_GB300_ERR_UNSUPPORTED
        assert "bytes of scratch" in lib.emsim_gb300_last_error().decode()
        assert not out.any()
    finally:
        lib.emsim_gb300_slice_plan_destroy(plan)
