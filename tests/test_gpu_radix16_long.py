"""Passes with 16 values per thread at lengths 512..4096 (pass tuning value 2): radix-16
Stockham passes then one radix-2/4/8 pass, rows synchronising per row, columns per CTA.

Against the FP64 oracle (relative L2 <= 1e-5, as for the radix-8 passes) through
multislice, space propagation, lens and the fused image; every tile choice gives
bitwise-identical waves; agreement with the radix-8 kernels within 1e-5.
"""
import numpy as np
import pytest

from oracle import multislice as om

pytestmark = pytest.mark.gpu

TOL = 1e-5
LONG = [512, 1024, 2048, 4096]


@pytest.fixture(scope="module")
def eng():
    import torch  # noqa: F401

    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import autotune, backend
    yield autotune, backend
    for n in LONG:
        autotune.set_tuning(n)


def _waves(rng, nb, n1, n2):
    return (rng.normal(size=(nb, n1, n2)) + 1j * rng.normal(size=(nb, n1, n2))).astype(np.complex64)


@pytest.mark.parametrize("n1,n2", [(512, 512), (1024, 1024), (2048, 2048), (4096, 4096), (512, 2048), (2048, 256),
                                   (1024, 4096)])
def test_multislice_against_fp64_and_radix8(eng, n1, n2):
    autotune, backend = eng
    rng = np.random.default_rng(n1 + 3 * n2)
    nb, ns = (2, 3) if n1 * n2 <= 1 << 21 else (1, 2)
    w = _waves(rng, nb, n1, n2)
    s = (rng.random((nb, ns, n1, n2)) * 30).astype(np.float32)
    wp = backend.WavePropagator(n1, n2, 0.1, 0.1, 300.0)
    try:
        for n in {n1, n2}:
            autotune.set_tuning(n, -1, 0, -1, 0)
        ref8 = wp.multislice_propagate(w, s, 0.5).get()
        for n in {n1, n2}:
            autotune.set_tuning(n, 2, 0, 2, 0)
        got = wp.multislice_propagate(w, s, 0.5).get()
    finally:
        for n in {n1, n2}:
            autotune.set_tuning(n)
    o64 = om.WavePropagator(n1, n2, 0.1, 0.1, 300.0, "fftw", np.float64)
    for i in range(nb):
        ref = o64.multislice_propagate(w[i].astype(np.complex128), s[i].astype(np.float64), 0.5)
        err = om.rel_l2(got[i], ref)
        assert err < TOL, (i, err)
    assert om.rel_l2(got, ref8) < TOL


@pytest.mark.parametrize("n", [512, 2048])
def test_tiles_bitwise_identical(eng, n):
    autotune, backend = eng
    rng = np.random.default_rng(n)
    nb = 4 if n == 512 else 1
    w = _waves(rng, nb, n, n)
    s = (rng.random((nb, 2, n, n)) * 30).astype(np.float32)
    wp = backend.WavePropagator(n, n, 0.1, 0.1, 300.0)
    T = n // 16
    ref = None
    try:
        for rows, cols in [(0, 0), (max(1, 128 // T), max(2, 256 // T)), (1, 2)]:
            autotune.set_tuning(n, 2, rows, 2, cols)
            got = wp.multislice_propagate(w, s, 0.5).get()
            if ref is None:
                ref = got
            np.testing.assert_array_equal(got, ref)
    finally:
        autotune.set_tuning(n)


def test_image_lens_space_2048(eng):
    autotune, backend = eng
    n, d, kev = 2048, 0.1, 300.0
    rng = np.random.default_rng(2048)
    sl = (np.abs(rng.normal(size=(3, n, n))) * 3).astype(np.float32)
    w = _waves(rng, 1, n, n)[0]
    wp = backend.WavePropagator(n, n, d, d, kev)
    o64 = om.WavePropagator(n, n, d, d, kev, "fftw", np.float64)
    try:
        autotune.set_tuning(n, 2, 0, 2, 0)
        img = np.asarray(wp.image(sl, 0.5, 20.0, 1.0, [400.0, 700.0], 0.02).get())
        lens = np.asarray(wp.lens_propagate(w, 1.0, 500.0, 0.02).get())
        space = np.asarray(wp.space_propagate(w, 0.5).get())
    finally:
        autotune.set_tuning(n)
    psi = o64.multislice_propagate(o64.init_wave(20.0).astype(np.complex128), sl.astype(np.float64), 0.5)
    for b, df in enumerate([400.0, 700.0]):
        assert om.rel_l2(img[b], om.intensity(o64.lens_propagate(psi, 1.0, df, 0.02))) < TOL
    assert om.rel_l2(lens, o64.lens_propagate(w, 1.0, 500.0, 0.02)) < TOL
    assert om.rel_l2(space, o64.space_propagate(w, 0.5)) < TOL


@pytest.mark.parametrize("n,zs,n_atoms", [(512, [6, 7, 8, 16], 4000), (1024, [6, 8], 12000), (2048, [6], 30000),
                                          (2048, [6, 8], 9000), (4096, [6], 12000)])
def test_slice_build_columns(eng, n, zs, n_atoms):
    """The slice build with the zero column tiles outside the filters' support (at pixel
    0.1 A the scattering factors end at |k| = 4 / A, inside Nyquist), against the FP64
    oracle, with the wave passes' tuning at either value (the build keeps its own
    column kernel).  The persistent column pass takes its 8-value form with per-row sums
    at 512 and 1024 and for planes above 6,144 atoms per slice pair (2048, 30,000 atoms
    in 3 pairs), its 16-value form with per-atom sums from 2048 otherwise."""
    autotune, backend = eng
    rng = np.random.default_rng(n + len(zs))
    d, dz, ns = 0.1, 0.5, 5
    xyz = ((rng.random((n_atoms, 3)) - 0.5) * np.array([ns * dz, n * d, n * d])).astype(np.float32)
    el = rng.choice(np.array(zs), size=n_atoms)
    order = np.argsort(el, kind="stable")
    xyz = xyz[order]
    counts = np.array([(el == z).sum() for z in sorted(zs)])
    b = backend.MultiSlicesBuilder(sorted(zs), ns, n, n, dz, d, d)
    try:
        autotune.set_tuning(n, -1, 0, -1, 0)
        ref8 = backend.build_slices_batch(b, [(xyz, counts)]).get()[0]
        autotune.set_tuning(n, -1, 0, 2, 0)
        got = backend.build_slices_batch(b, [(xyz, counts)]).get()[0]
    finally:
        autotune.set_tuning(n)
    hist = om.bin_atoms_cuda(xyz, counts, (ns, n, n), (dz, d, d)).astype(np.float64)
    ref = om.make_slices(hist, om.scattering_factors_half(sorted(zs), n, n, d, d), "fftw", np.float64)
    assert om.rel_l2(got, ref) < TOL
    assert om.rel_l2(got, ref8) < TOL
