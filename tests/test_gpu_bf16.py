"""Split-BF16 tensor-core passes (precision mode "bf16x3") against the FP64 oracle,
through the C ABI.

Tolerance: relative L2 <= TOL = 1e-4 per wave and per image against FP64 (the split
keeps about 16 significant bits per 16-point stage, accumulated in fp32); results are
bitwise reproducible; sizes without a tensor-core pass are unchanged by the mode.
"""
import numpy as np
import pytest

from oracle import multislice as om

pytestmark = pytest.mark.gpu

TOL = 1e-4


@pytest.fixture(scope="module")
def eng():
    import torch  # noqa: F401

    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import backend
    yield backend
    backend.set_precision("fp32")


def _rand_wave(rng, shape):
    return (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)


def test_precision_switch(eng):
    from emsim_gb300 import _native
    assert eng.get_precision() == "fp32"
    eng.set_precision("bf16x3")
    assert eng.get_precision() == "bf16x3"
    eng.set_precision("fp32")
    assert eng.get_precision() == "fp32"
    with pytest.raises(ValueError):
        eng.set_precision("fp16")
    with pytest.raises(_native.NativeError):
        _native.call("emsim_gb300_set_precision", 7)
    assert eng.get_precision() == "fp32"


@pytest.mark.parametrize("d", [0.5, 1.0])
def test_multislice_bf16_matches_fp64(eng, d):
    n, ns, nb, dz, kev = 256, 6, 3, 1.0, 300.0
    rng = np.random.default_rng(int(d * 10))
    w = _rand_wave(rng, (nb, n, n))
    sl = (np.abs(rng.normal(size=(ns, n, n))) * 3).astype(np.float32)
    wp = eng.WavePropagator(n, n, d, d, kev)
    eng.set_precision("fp32")
    ref32 = np.asarray(wp.multislice_propagate(w, sl, dz).get())
    eng.set_precision("bf16x3")
    try:
        got = np.asarray(wp.multislice_propagate(w, sl, dz).get())
        again = np.asarray(wp.multislice_propagate(w, sl, dz).get())
    finally:
        eng.set_precision("fp32")
    np.testing.assert_array_equal(got, again)
    o64 = om.WavePropagator(n, n, d, d, kev, "fftw", np.float64)
    for b in range(nb):
        ref = o64.multislice_propagate(w[b], sl, dz)
        e = om.rel_l2(got[b], ref)
        print(f"\nbf16x3 multislice n={n} d={d} wave {b}: rel-L2 vs FP64 {e:.3e}, "
              f"fp32 {om.rel_l2(ref32[b], ref):.3e}")
        assert e < TOL
    # the mode is in effect: the result differs from the FP32 passes
    assert 0 < om.rel_l2(got, ref32) < TOL


def test_image_bf16_blob_matches_fp64(eng):
    """A 20,000-atom blob through binning, slice build and the fused image with the
    tensor-core multislice passes, against the FP64 oracle."""
    n, d, dz, kev, cs, dose = 256, 1.0, 2.0, 300.0, 1.0, 20.0
    zs = [6, 7, 8, 16]
    el, xyz0 = om.protein_blob(20_000, radius=30.0, seed=3)
    _, xyz, _, cnt = om.sort_elements_and_count(el, xyz0, zs)
    ns = int(np.ceil(2 * 30.0 / dz)) + 2
    from emsim_gb300 import physics
    lam = physics.electron_wave_length_angstrom(kev)
    df, ap = physics.scherzer_condition(lam, cs)
    b = eng.MultiSlicesBuilder(zs, ns, n, n, dz, d, d)
    slices = eng.build_slices_batch(b, [(xyz, cnt)])
    wp = eng.WavePropagator(n, n, d, d, kev)
    eng.set_precision("bf16x3")
    try:
        img = np.asarray(wp.image(slices[0], dz, dose, cs, df, ap).get())
    finally:
        eng.set_precision("fp32")
    img32 = np.asarray(wp.image(slices[0], dz, dose, cs, df, ap).get())
    v64 = np.asarray(slices.get())[0].astype(np.float64)
    o64 = om.WavePropagator(n, n, d, d, kev, "fftw", np.float64)
    psi = o64.multislice_propagate(o64.init_wave(dose).astype(np.complex128), v64, dz)
    ref = om.intensity(o64.lens_propagate(psi, cs, df, ap))
    e, e32 = om.rel_l2(img, ref), om.rel_l2(img32, ref)
    ec = om.rel_l2(img - img.mean(), ref - ref.mean())
    print(f"\nbf16x3 image, 20k-atom blob, {ns} slices: rel-L2 vs FP64 {e:.3e} (contrast {ec:.3e}); fp32 {e32:.3e}")
    assert e < TOL


def test_other_sizes_unchanged_in_bf16_mode(eng):
    from emsim_gb300 import _native
    n, ns, dz = 128, 5, 1.0
    rng = np.random.default_rng(5)
    w = _rand_wave(rng, (2, n, n))
    sl = (np.abs(rng.normal(size=(ns, n, n))) * 3).astype(np.float32)
    wp = eng.WavePropagator(n, n, 0.5, 0.5, 200.0)
    ref = np.asarray(wp.multislice_propagate(w, sl, dz).get())
    eng.set_precision("bf16x3")
    try:
        got = np.asarray(wp.multislice_propagate(w, sl, dz).get())
    finally:
        eng.set_precision("fp32")
    np.testing.assert_array_equal(got, ref)
    assert _native.check_device_error() == 0


@pytest.mark.parametrize("n1,n2", [(256, 128), (128, 256), (256, 512)])
def test_rectangular_waves_mix_bf16_and_fp32_passes(eng, n1, n2):
    """A side of 256 runs its pass on the tensor cores, the other side stays FP32."""
    ns, dz, d = 5, 1.5, 0.5
    rng = np.random.default_rng(n1 + 3 * n2)
    w = _rand_wave(rng, (2, n1, n2))
    sl = (np.abs(rng.normal(size=(ns, n1, n2))) * 3).astype(np.float32)
    wp = eng.WavePropagator(n1, n2, d, d, 200.0)
    ref32 = np.asarray(wp.multislice_propagate(w, sl, dz).get())
    eng.set_precision("bf16x3")
    try:
        got = np.asarray(wp.multislice_propagate(w, sl, dz).get())
    finally:
        eng.set_precision("fp32")
    o64 = om.WavePropagator(n1, n2, d, d, 200.0, "fftw", np.float64)
    for b in range(2):
        assert om.rel_l2(got[b], o64.multislice_propagate(w[b], sl, dz)) < TOL
    assert 0 < om.rel_l2(got, ref32) < TOL
