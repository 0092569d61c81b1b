"""The radix-16 passes of length 256 (pass tuning value 2) through the public paths:
fused images, lens, space propagation, ragged images and the adjoint, against the FP64
oracle, with the tuning forced on.

Tolerances as for the radix-8 passes: relative L2 <= 1e-5 (waves, images), 2e-5
(gradients against the FP64 adjoint).
"""
import numpy as np
import pytest

from oracle import multislice as om
from oracle.adjoint import ImageChain

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def eng():
    import torch  # noqa: F401

    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import autotune, backend
    autotune.set_tuning(256, 2, 0, 2, 8)
    yield backend
    autotune.set_tuning(256)


def test_image_lens_space(eng):
    n, d, kev = 256, 0.5, 300.0
    rng = np.random.default_rng(16)
    sl = (np.abs(rng.normal(size=(5, n, n))) * 3).astype(np.float32)
    w = (rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))).astype(np.complex64)
    wp = eng.WavePropagator(n, n, d, d, kev)
    o64 = om.WavePropagator(n, n, d, d, kev, "fftw", np.float64)
    img = np.asarray(wp.image(sl, 1.5, 20.0, 1.3, [500.0, 900.0], 0.012).get())
    psi = o64.multislice_propagate(o64.init_wave(20.0).astype(np.complex128), sl.astype(np.float64), 1.5)
    for b, df in enumerate([500.0, 900.0]):
        assert om.rel_l2(img[b], om.intensity(o64.lens_propagate(psi, 1.3, df, 0.012))) < TOL
    assert om.rel_l2(np.asarray(wp.lens_propagate(w, 1.3, 700.0, 0.012).get()),
                     o64.lens_propagate(w, 1.3, 700.0, 0.012)) < TOL
    assert om.rel_l2(np.asarray(wp.space_propagate(w, 2.0).get()), o64.space_propagate(w, 2.0)) < TOL


def test_ragged_images_match_single(eng):
    n = 256
    rng = np.random.default_rng(5)
    stacks = (np.abs(rng.normal(size=(3, 6, n, n))) * 3).astype(np.float32)
    counts = [6, 3, 5]
    wp = eng.WavePropagator(n, n, 0.5, 0.5, 200.0)
    got = np.asarray(eng.image_ragged(wp, stacks, counts, 1.5, 20.0, 1.3, [600.0, 700.0, 800.0], 0.012).get())
    for i, (c, df) in enumerate(zip(counts, [600.0, 700.0, 800.0])):
        one = np.asarray(wp.image(stacks[i, :c], 1.5, 20.0, 1.3, df, 0.012).get())
        np.testing.assert_array_equal(got[i], one)


def test_adjoint_gradient(eng):
    import torch
    from emsim_gb300 import autograd
    n, ns = 256, 6
    rng = np.random.default_rng(21)
    v = torch.tensor(rng.uniform(0, 120, size=(ns, n, n)).astype(np.float32), device="cuda", requires_grad=True)
    dfs = [500.0, 900.0]
    wp = eng.WavePropagator(n, n, 0.5, 0.5, 200.0)
    target = torch.tensor(rng.uniform(15, 25, size=(2, n, n)).astype(np.float32), device="cuda")
    img = autograd.image(wp, v, 1.0, 20.0, 1.3, dfs, 10e-3)
    loss = torch.mean((img - target) ** 2)
    loss.backward()
    g = (2.0 * (img.detach() - target) / img.numel()).cpu().numpy().astype(np.float64)
    chain = ImageChain(n, n, 0.5, 0.5, 200.0)
    g64 = chain.adjoint(v.detach().cpu().numpy(), 1.0, 20.0, 1.3, dfs, 10e-3, 2, g)
    assert om.rel_l2(v.grad.cpu().numpy(), g64) < 2e-5
