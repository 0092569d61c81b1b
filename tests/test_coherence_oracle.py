"""CPU checks of the partial-coherence oracle (oracle/coherence.py) and of the host-side
quadrature the package uses.  Parity against the reference is unpinned: the reference
has no partial coherence (its README lists it as future work)."""
import math

import numpy as np
import pytest

from oracle import coherence as oc
from oracle import multislice as om


@pytest.mark.parametrize("n", [1, 3, 7, 12])
def test_quadrature_moments(n):
    df, sig = 700.0, 45.0
    x, w = oc.quadrature(df, sig, n)
    assert np.isclose(w.sum(), 1.0, rtol=1e-14)
    assert np.isclose(np.sum(w * x), df, rtol=1e-14)
    if n >= 2:
        assert np.isclose(np.sum(w * (x - df) ** 2), sig * sig, rtol=1e-12)


def test_package_quadrature_matches_oracle():
    from emsim_gb300 import backend
    for sig in (0.0, 20.0):
        a = backend.focal_spread_quadrature(500.0, sig, 9)
        b = oc.quadrature(500.0, sig, 9)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
    with pytest.raises(ValueError):
        backend.focal_spread_quadrature(500.0, -1.0)


def _wave(n1, n2, seed=0):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(n1, n2)) + 1j * rng.normal(size=(n1, n2))


def test_coherent_limit_equals_lens_intensity():
    wp = om.WavePropagator(64, 48, 0.5, 0.5, 200.0, "fftw", np.float64)
    psi = _wave(64, 48)
    got = oc.lens_intensity_incoherent(wp, psi, 1.3, [700.0], [1.0], 12e-3, 0.0)
    ref = om.intensity(wp.lens_propagate(psi, 1.3, 700.0, 12e-3))
    np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_spatial_envelope_properties():
    wp = om.WavePropagator(64, 64, 0.5, 0.5, 300.0, "fftw", np.float64)
    e0 = oc.spatial_envelope(wp, 1.0, 600.0, 0.0)
    assert np.all(e0 == 1.0)
    e1 = oc.spatial_envelope(wp, 1.0, 600.0, 0.5e-3)
    e2 = oc.spatial_envelope(wp, 1.0, 600.0, 1.0e-3)
    assert e1[0, 0] == 1.0 and np.all(e1 <= 1.0) and np.all(e2 <= e1)
    # the closed form at one frequency
    lam = wp.wave_length
    k2 = wp.f2[3, 5]
    g = 1.0 * 1e7 * lam ** 3 * k2 - 600.0 * lam
    assert math.isclose(e1[3, 5], math.exp(-(math.pi * 0.5e-3 / lam) ** 2 * k2 * g * g), rel_tol=1e-14)


def test_partial_coherence_reduces_contrast():
    """Focal spread and beam divergence damp high-frequency contrast of a weak-phase wave."""
    n = 64
    wp = om.WavePropagator(n, n, 0.5, 0.5, 200.0, "fftw", np.float64)
    rng = np.random.default_rng(3)
    psi = np.exp(1j * 0.05 * rng.normal(size=(n, n)))
    coh = oc.lens_intensity_incoherent(wp, psi, 1.3, [700.0], [1.0], 20e-3)
    dfs, wts = oc.quadrature(700.0, 80.0, 9)
    part = oc.lens_intensity_incoherent(wp, psi, 1.3, dfs, wts, 20e-3, 1e-3)
    assert np.std(part) < np.std(coh)
    assert np.isclose(part.mean(), coh.mean(), rtol=0.05)
