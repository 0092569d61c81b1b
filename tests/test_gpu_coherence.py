"""Partially coherent imaging on the GPU (emsim_gb300_lens_intensity_incoherent and the
Pipe / TEM integration) against the FP64 oracle of oracle/coherence.py, through the C
ABI.  The reference has no partial coherence, so parity is against the published
formulas restated in FP64 (unpinned against the reference).

Tolerances: relative L2 <= TOL = 1e-5 against FP64; the coherent limit (one defocus,
weight 1, no envelope) equals lens_propagate + intensity to 1e-6.
"""
import numpy as np
import pytest

from oracle import coherence as oc
from oracle import multislice as om

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.fixture(scope="module")
def eng():
    import torch  # noqa: F401

    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import backend
    return backend


def _waves(rng, nb, n1, n2):
    # exit-wave-like: unit modulus with a random phase, plus a little amplitude noise
    ph = rng.normal(scale=0.3, size=(nb, n1, n2))
    return ((1 + 0.05 * rng.normal(size=(nb, n1, n2))) * np.exp(1j * ph)).astype(np.complex64)


CASES = [(64, 64, 0.0, 0.0), (64, 64, 40.0, 0.0), (256, 256, 0.0, 0.5e-3), (256, 256, 30.0, 0.3e-3),
         (48, 40, 25.0, 0.4e-3), (128, 64, 60.0, 0.0)]


@pytest.mark.parametrize("n1,n2,spread,angle", CASES)
def test_lens_intensity_incoherent_matches_fp64(eng, n1, n2, spread, angle):
    rng = np.random.default_rng(n1 + 7 * n2)
    d, kev, cs, df, ap = 0.5, 300.0, 1.2, 650.0, 15e-3
    w = _waves(rng, 2, n1, n2)
    wp = eng.WavePropagator(n1, n2, d, d, kev)
    dfs, wts = eng.focal_spread_quadrature(df, spread, 7)
    got = np.asarray(wp.lens_intensity_incoherent(w, cs, dfs, wts, ap, angle).get())
    o64 = om.WavePropagator(n1, n2, d, d, kev, "fftw", np.float64)
    ref = oc.lens_intensity_incoherent(o64, w.astype(np.complex128), cs, dfs, wts, ap, angle)
    assert got.shape == (2, n1, n2)
    e = om.rel_l2(got, ref)
    assert e < TOL, e


def test_coherent_limit_equals_lens_and_intensity(eng):
    rng = np.random.default_rng(1)
    n = 128
    w = _waves(rng, 3, n, n)
    wp = eng.WavePropagator(n, n, 0.5, 0.5, 200.0)
    got = np.asarray(wp.lens_intensity_incoherent(w, 1.3, [700.0], [1.0], 12e-3).get())
    lensed = wp.lens_propagate(w, 1.3, 700.0, 12e-3)
    ref = np.asarray(eng.intensity(lensed).get())
    assert om.rel_l2(got, ref) < 1e-6


def test_image_partially_coherent_and_pipe(eng):
    """Slices -> multislice -> partially coherent lens through the backend and through
    Pipe.run / run_batch with a partially coherent TEM, against the FP64 chain."""
    from emsim_gb300 import atoms, pipe, tem
    el, xyz = om.protein_blob(3000, radius=12.0, seed=9)
    m = tem.TEM(electron_dose=20.0, beam_energy_kev=200.0, cs_mm=1.3, defocus=700.0, aperture=10e-3,
                focal_spread=50.0, illumination_angle=0.4e-3, n_focal=7)
    p = pipe.Pipe(m, resolution=1.0, slice_thickness=2.0, roi=128, add_water=False)
    mol = atoms.AtomList(el, xyz)
    img = np.asarray(p.run(mol).get())
    slices = np.asarray(p.build_slices(mol).get())
    ns, n1, n2 = slices.shape
    ref = oc.image_partially_coherent(n1, n2, 0.5, 0.5, 200.0, slices, 2.0, 20.0, 1.3, 700.0, 10e-3, 50.0, 0.4e-3, 7)
    assert om.rel_l2(img, ref) < TOL
    # the batch API gives the same images, and partial coherence changes the image
    both = p.run_batch([mol, mol], to_host=True)
    np.testing.assert_array_equal(both[0], img)
    np.testing.assert_array_equal(both[1], img)
    m.focal_spread, m.illumination_angle = 0.0, 0.0
    coherent = np.asarray(p.run(mol).get())
    assert om.rel_l2(coherent, img) > 1e-4
    assert np.std(img) < np.std(coherent)


def test_incoherent_rejects_bad_arguments(eng):
    from emsim_gb300 import _native
    wp = eng.WavePropagator(64, 64, 0.5, 0.5, 200.0)
    w = np.ones((64, 64), np.complex64)
    with pytest.raises(ValueError):
        wp.lens_intensity_incoherent(w, 1.3, [600.0, 700.0], [1.0], 10e-3)
    with pytest.raises(_native.NativeError):
        wp.lens_intensity_incoherent(w, 1.3, [700.0], [1.0], 10e-3, illumination_angle=-1e-3)
    assert _native.check_device_error() == 0
