"""Sides that are not powers of two run Bluestein line transforms on the power-of-two
fast path (csrc/bluestein.cu).  Waves, images and slices against the FFTW-semantics FP32
restatement and the FP64 oracle, through the C ABI.

Tolerance: relative L2 <= 1e-5, as for the power-of-two sizes.  Propagated waves are
compared with the FP32 restatement: on some grids (300 x 300 at 0.4 or 0.5 A) a
frequency lies within float32 rounding of the 2/3 band-limit, which the reference
evaluates in float32 (kept) and FP64 classifies the other way, so FP64 differs there by
the energy of those few coefficients; lens and slices are compared with FP64 too.
"""
import numpy as np
import pytest

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


def _np(t):
    return t.get() if hasattr(t, "get") else np.asarray(t)


SIZES = [(300, 300), (97, 97), (384, 200), (6, 10), (2047, 3), (1000, 24)]


@pytest.mark.parametrize("n1,n2", SIZES)
def test_waves_lens_multislice(eng, n1, n2):
    rng = np.random.default_rng(n1 * 3 + n2)
    d = 0.4
    w = (rng.normal(size=(2, n1, n2)) + 1j * rng.normal(size=(2, n1, n2))).astype(np.complex64)
    sl = (np.abs(rng.normal(size=(3, n1, n2))) * 3).astype(np.float32)
    wp = eng.WavePropagator(n1, n2, d, d, 300.0)
    o32 = om.WavePropagator(n1, n2, d, d, 300.0, "fftw", np.float32)
    o64 = om.WavePropagator(n1, n2, d, d, 300.0, "fftw", np.float64)
    got = _np(wp.multislice_propagate(w, sl, 1.5))
    for b in range(2):
        assert om.rel_l2(got[b], o32.multislice_propagate(w[b], sl, 1.5)) < TOL
    got = _np(wp.lens_propagate(w[0], 1.3, 700.0, 0.012))
    assert om.rel_l2(got, o64.lens_propagate(w[0], 1.3, 700.0, 0.012)) < TOL
    assert om.rel_l2(got, o32.lens_propagate(w[0], 1.3, 700.0, 0.012)) < TOL
    img = _np(wp.image(sl, 1.5, 20.0, 1.3, [600.0, 800.0], 0.012))
    psi = o32.multislice_propagate(o32.init_wave(20.0), sl, 1.5)
    for b, df in enumerate([600.0, 800.0]):
        assert om.rel_l2(img[b], om.intensity(o32.lens_propagate(psi, 1.3, df, 0.012))) < TOL


def test_slices_generic_side(eng):
    zs, ns, n, dz, d = [6, 8, 29], 4, 300, 2.0, 0.5
    rng = np.random.default_rng(4)
    el = rng.choice(np.array(zs), size=800)
    xyz = ((rng.random((800, 3)) * 2 - 1) * np.array([ns * dz / 2, n * d / 2, n * d / 2]) * 0.9).astype(np.float32)
    _, xyz_s, _, cnt = om.sort_elements_and_count(el, xyz, zs)
    b = eng.MultiSlicesBuilder(zs, ns, n, n, dz, d, d)
    hist = b.bin_atoms_multi_slices(xyz_s, cnt)
    got = _np(b.make_multi_slices(hist))
    sf = om.scattering_factors_half(zs, n, n, d, d)
    ref = om.make_slices(_np(hist).astype(np.float64), sf, "fftw", np.float64)
    assert om.rel_l2(got, ref) < TOL


def test_generic_side_is_deterministic(eng):
    rng = np.random.default_rng(8)
    n1, n2 = 300, 150
    w = (rng.normal(size=(n1, n2)) + 1j * rng.normal(size=(n1, n2))).astype(np.complex64)
    wp = eng.WavePropagator(n1, n2, 0.5, 0.5, 200.0)
    a = _np(wp.space_propagate(w, 2.0))
    b = _np(wp.space_propagate(w, 2.0))
    np.testing.assert_array_equal(a, b)
