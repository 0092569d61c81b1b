"""GPU adjoint multislice (checkpointed forward + conjugate sweep) against the FP64
adjoint oracle and FP64 central differences, through the C ABI and the autograd
Function.

Tolerances: the checkpointed image equals the fused image to relative L2 1e-6; the
float32 gradient dLoss/dV matches the FP64 adjoint to relative L2 ADJ_TOL and FP64
central differences (directional derivatives) to FD_TOL; gradients do not depend on the
checkpoint spacing (bitwise).
"""
import ctypes

import numpy as np
import pytest

from oracle import multislice as om
from oracle.adjoint import ImageChain, loss_weighted

pytestmark = pytest.mark.gpu

ADJ_TOL = 2e-5
FD_TOL = 2e-5


@pytest.fixture(scope="module")
def eng():
    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import autograd, backend
    return backend, autograd


def _grad_native(backend, wp, slices, dz, dose, cs, dfs, ap, nb, g, every):
    """(image, dLoss/dV) straight through the two C-ABI entry points."""
    import torch
    from emsim_gb300 import _native
    n1, n2 = wp.wave_shape
    s = torch.as_tensor(slices, device="cuda").contiguous()
    ns, stride = (s.shape[1], s.shape[1] * n1 * n2) if s.dim() == 4 else (s.shape[0], 0)
    lib = _native.load()
    n_ck = lib.emsim_gb300_adjoint_checkpoints(ns, every)
    img = torch.empty((nb, n1, n2), dtype=torch.float32, device="cuda")
    u = torch.empty((nb, n1, n2), dtype=torch.complex64, device="cuda")
    ck = torch.empty((max(n_ck, 1), nb, n1, n2), dtype=torch.complex64, device="cuda")
    d = np.ascontiguousarray(np.atleast_1d(np.asarray(dfs, np.float64)))
    dp = d.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    st = backend._stream()
    _native.call("emsim_gb300_multislice_image_ckpt", wp._plan.handle, backend._ptr(s), ns, stride, dz, dose, cs, dp,
                 len(d), ap, backend._ptr(img), backend._ptr(u), backend._ptr(ck), every, nb, st)
    gt = torch.as_tensor(np.asarray(g, np.float32), device="cuda").contiguous()
    nbytes = lib.emsim_gb300_adjoint_workspace_size(wp._plan.handle, ns, every, nb, stride)
    work = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    grad = torch.empty_like(s)
    _native.call("emsim_gb300_multislice_image_adjoint", wp._plan.handle, backend._ptr(s), ns, stride, dz, dose, cs,
                 dp, len(d), ap, backend._ptr(gt), backend._ptr(u), backend._ptr(ck), every, backend._ptr(grad),
                 backend._ptr(work), nbytes, nb, st)
    torch.cuda.synchronize()
    return img.cpu().numpy(), grad.cpu().numpy()


def _case(n, ns, nb, per_image, seed):
    rng = np.random.default_rng(seed)
    shape = (nb, ns, n, n) if per_image else (ns, n, n)
    v = rng.uniform(0.0, 150.0, size=shape).astype(np.float32)
    w = rng.standard_normal((nb, n, n)).astype(np.float32)
    dfs = rng.uniform(300.0, 1500.0, size=nb)
    return v, w, dfs


CASES = [(64, 7, 3, False), (64, 5, 2, True), (256, 16, 2, False), (128, 9, 1, False), (32, 4, 4, True)]


@pytest.mark.parametrize("n,ns,nb,per_image", CASES)
def test_adjoint_matches_fp64_oracle(eng, n, ns, nb, per_image):
    backend, _ = eng
    d, kev, dz, dose, cs, ap = 0.5, 200.0, 1.0, 20.0, 1.3, 12e-3
    v, w, dfs = _case(n, ns, nb, per_image, seed=n + ns + nb)
    wp = backend.WavePropagator(n, n, d, d, kev)
    every = max(1, int(np.ceil(np.sqrt(ns))))
    img, grad = _grad_native(backend, wp, v, dz, dose, cs, dfs, ap, nb, w, every)
    chain = ImageChain(n, n, d, d, kev)
    img64 = chain.forward(v, dz, dose, cs, dfs, ap, nb)
    assert om.rel_l2(img, img64) < 1e-5
    fused = backend.WavePropagator(n, n, d, d, kev).image(v, dz, dose, cs, list(dfs), ap, n_batch=nb)
    assert om.rel_l2(img, np.asarray(fused.get()).reshape(img.shape)) < 1e-6
    g64 = chain.adjoint(v, dz, dose, cs, dfs, ap, nb, w)
    err = om.rel_l2(grad, g64)
    assert grad.shape == v.shape
    assert err < ADJ_TOL, err


def test_adjoint_central_differences(eng):
    backend, _ = eng
    n, ns, nb = 64, 6, 2
    d, kev, dz, dose, cs, ap = 0.5, 300.0, 1.5, 20.0, 1.0, 15e-3
    v, w, dfs = _case(n, ns, nb, False, seed=42)
    wp = backend.WavePropagator(n, n, d, d, kev)
    _, grad = _grad_native(backend, wp, v, dz, dose, cs, dfs, ap, nb, w, every=2)
    chain = ImageChain(n, n, d, d, kev)
    rng = np.random.default_rng(9)
    v64 = v.astype(np.float64)
    for _ in range(3):
        dv = rng.standard_normal(v.shape)
        h = 1e-3
        lp = loss_weighted(chain.forward(v64 + h * dv, dz, dose, cs, dfs, ap, nb), w)
        lm = loss_weighted(chain.forward(v64 - h * dv, dz, dose, cs, dfs, ap, nb), w)
        fd = (lp - lm) / (2 * h)
        an = float(np.sum(grad.astype(np.float64) * dv))
        assert abs(fd - an) <= FD_TOL * abs(fd), (fd, an)


def test_gradient_independent_of_checkpoint_spacing(eng):
    backend, _ = eng
    n, ns, nb = 64, 10, 2
    v, w, dfs = _case(n, ns, nb, False, seed=5)
    wp = backend.WavePropagator(n, n, 0.5, 0.5, 200.0)
    ref_img, ref = _grad_native(backend, wp, v, 2.0, 20.0, 1.3, dfs, 10e-3, nb, w, every=1)
    for every in (2, 3, 4, 9, 10, 25):
        img, g = _grad_native(backend, wp, v, 2.0, 20.0, 1.3, dfs, 10e-3, nb, w, every=every)
        np.testing.assert_array_equal(img, ref_img)
        np.testing.assert_array_equal(g, ref)


def test_shared_stack_is_ordered_sum_of_image_gradients(eng):
    backend, _ = eng
    n, ns, nb = 64, 5, 3
    v, w, dfs = _case(n, ns, nb, False, seed=8)
    wp = backend.WavePropagator(n, n, 0.5, 0.5, 200.0)
    _, g_shared = _grad_native(backend, wp, v, 2.0, 20.0, 1.3, dfs, 10e-3, nb, w, every=2)
    v4 = np.ascontiguousarray(np.broadcast_to(v, (nb,) + v.shape))
    _, g4 = _grad_native(backend, wp, v4, 2.0, 20.0, 1.3, dfs, 10e-3, nb, w, every=2)
    acc = np.zeros_like(g_shared)
    for i in range(nb):
        acc = (acc + g4[i]).astype(np.float32)
    np.testing.assert_array_equal(g_shared, acc)


def test_autograd_function_mse(eng):
    import torch
    backend, autograd = eng
    n, ns = 128, 8
    rng = np.random.default_rng(21)
    v = torch.tensor(rng.uniform(0, 120, size=(ns, n, n)).astype(np.float32), device="cuda", requires_grad=True)
    dfs = [500.0, 900.0, 1300.0]
    wp = backend.WavePropagator(n, n, 0.5, 0.5, 200.0)
    target = torch.tensor(rng.uniform(15, 25, size=(3, n, n)).astype(np.float32), device="cuda")
    img = autograd.image(wp, v, 1.0, 20.0, 1.3, dfs, 10e-3)
    loss = torch.mean((img - target) ** 2)
    loss.backward()
    g = (2.0 * (img.detach() - target) / img.numel()).cpu().numpy().astype(np.float64)
    chain = ImageChain(n, n, 0.5, 0.5, 200.0)
    g64 = chain.adjoint(v.detach().cpu().numpy(), 1.0, 20.0, 1.3, dfs, 10e-3, 3, g)
    assert om.rel_l2(v.grad.cpu().numpy(), g64) < ADJ_TOL
    # per-image stacks
    v4 = v.detach().unsqueeze(0).repeat(3, 1, 1, 1).requires_grad_(True)
    img4 = autograd.image(wp, v4, 1.0, 20.0, 1.3, dfs, 10e-3)
    torch.mean((img4 - target) ** 2).backward()
    assert v4.grad.shape == v4.shape
    assert om.rel_l2(v4.grad.sum(0).cpu().numpy(), v.grad.cpu().numpy()) < 1e-6


def test_adjoint_rejects_bad_arguments(eng):
    import torch
    backend, autograd = eng
    from emsim_gb300 import _native
    wp = backend.WavePropagator(48, 48, 0.5, 0.5, 200.0)  # not a power of two
    v = torch.zeros((3, 48, 48), device="cuda", requires_grad=True)
    with pytest.raises(_native.NativeError):
        autograd.image(wp, v, 1.0, 20.0, 1.3, [700.0], 10e-3)
    assert _native.load().emsim_gb300_adjoint_checkpoints(0, 3) == 0
    assert _native.load().emsim_gb300_adjoint_checkpoints(10, 3) == 3
    assert _native.check_device_error() == 0
