"""GPU parity of every engine entry point against the oracle (FFTW/CUDA FP32 semantics
restated in numpy; FP64 for accuracy), through the C ABI.

Tolerances: bit-exact for binning (integer counts); relative L2 <= 1e-5 for float32
waves, slices and images against the FP32 restatement and the FP64 oracle.
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


def _rand_wave(rng, shape):
    return (rng.normal(size=shape) + 1j * rng.normal(size=shape)).astype(np.complex64)


SIZES = [(64, 64), (256, 256), (512, 512), (64, 128), (128, 32), (48, 40), (30, 30), (8, 16)]


@pytest.mark.parametrize("n1,n2", SIZES)
def test_space_propagate(eng, n1, n2):
    rng = np.random.default_rng(n1 * 7 + n2)
    d = 0.4
    w = _rand_wave(rng, (n1, n2))
    wp = eng.WavePropagator(n1, n2, d, d * 1.1, 200.0)
    got = _np(wp.space_propagate(w, 2.0))
    ref = om.WavePropagator(n1, n2, d, d * 1.1, 200.0, "fftw", np.float32).space_propagate(w, 2.0)
    r64 = om.WavePropagator(n1, n2, d, d * 1.1, 200.0, "fftw", np.float64).space_propagate(w, 2.0)
    assert om.rel_l2(got, ref) < TOL
    assert om.rel_l2(got, r64) < TOL


@pytest.mark.parametrize("n1,n2", SIZES)
def test_transmit_single_multi_lens(eng, n1, n2):
    rng = np.random.default_rng(n1 + 3 * n2)
    d = 0.5
    w = _rand_wave(rng, (n1, n2))
    sl = (np.abs(rng.normal(size=(4, n1, n2))) * 3).astype(np.float32)
    wp = eng.WavePropagator(n1, n2, d, d, 300.0)
    o32 = om.WavePropagator(n1, n2, d, d, 300.0, "fftw", np.float32)
    o64 = om.WavePropagator(n1, n2, d, d, 300.0, "fftw", np.float64)
    for name, args in [("slice_transmit", (w, sl[0])), ("singleslice_propagate", (w, sl[0], 1.5)),
                       ("multislice_propagate", (w, sl, 1.5)), ("lens_propagate", (w, 1.3, 700.0, 0.012))]:
        got = _np(getattr(wp, name)(*args))
        assert om.rel_l2(got, getattr(o32, name)(*args)) < TOL, name
        assert om.rel_l2(got, getattr(o64, name)(*args)) < TOL, name


def test_init_wave_and_intensity_exact(eng):
    wp = eng.WavePropagator(64, 32, 0.3, 0.3, 200.0)
    w = _np(wp.init_wave(20.0))
    np.testing.assert_array_equal(w, om.WavePropagator(64, 32, 0.3, 0.3, 200.0).init_wave(20.0))
    x = _rand_wave(np.random.default_rng(0), (3, 17, 5))
    got = _np(eng.intensity(x))
    np.testing.assert_array_equal(got, (x.real * x.real + x.imag * x.imag).astype(np.float32))


def test_multislice_edge_cases(eng):
    rng = np.random.default_rng(11)
    wp = eng.WavePropagator(64, 64, 0.5, 0.5, 200.0)
    w = _rand_wave(rng, (64, 64))
    # zero slices: the wave passes unchanged (the numpy path's loop runs zero times)
    np.testing.assert_array_equal(_np(wp.multislice_propagate(w, np.zeros((0, 64, 64), np.float32), 2.0)), w)
    # one slice == singleslice
    sl = rng.random((1, 64, 64)).astype(np.float32)
    a = _np(wp.multislice_propagate(w, sl, 2.0))
    b = _np(wp.singleslice_propagate(w, sl[0], 2.0))
    assert om.rel_l2(a, b) < 1e-6
    with pytest.raises(ValueError):
        wp.space_propagate(np.zeros((32, 64), np.complex64), 1.0)


def test_batch_equals_single(eng):
    rng = np.random.default_rng(12)
    n = 128
    wp = eng.WavePropagator(n, n, 0.5, 0.5, 200.0)
    ws = _rand_wave(rng, (3, n, n))
    sl = rng.random((3, 5, n, n)).astype(np.float32)
    batch = _np(wp.multislice_propagate(ws, sl, 2.0))
    for b in range(3):
        one = _np(wp.multislice_propagate(ws[b], sl[b], 2.0))
        np.testing.assert_array_equal(batch[b], one)


def test_determinism(eng):
    rng = np.random.default_rng(13)
    wp = eng.WavePropagator(256, 256, 0.5, 0.5, 200.0)
    w = _rand_wave(rng, (256, 256))
    sl = rng.random((6, 256, 256)).astype(np.float32)
    a = _np(wp.multislice_propagate(w, sl, 2.0))
    b = _np(wp.multislice_propagate(w, sl, 2.0))
    np.testing.assert_array_equal(a, b)


# ---------------------------------------------------------------------------------
# binning: bit-exact
# ---------------------------------------------------------------------------------
BIN_CASES = [((24, 30), (0.5, 0.4)), ((25, 31), (0.5, 0.4)), ((6, 16, 20), (1.3, 0.5, 0.45)),
             ((7, 17, 21), (1.3, 0.5, 0.45)), ((40, 256, 256), (2.0, 1.0, 1.0))]


@pytest.mark.parametrize("shape,steps", BIN_CASES)
def test_binning_bit_exact(eng, shape, steps):
    rng = np.random.default_rng(len(shape) * 1000 + shape[-1])
    half = [n * d / 2 * 1.15 for n, d in zip(shape, steps)]
    if len(shape) == 2:
        half = [1.0] + half
    n = 5000
    el = rng.choice(np.array([1, 6, 7, 8, 16, 29]), size=n)
    xyz = ((rng.random((n, 3)) * 2 - 1) * np.array(half)).astype(np.float32)
    # atoms exactly on both CUDA-rule edges of every binned axis
    edge = []
    axes = (1, 2) if len(shape) == 2 else (0, 1, 2)
    for ax, nn, d in zip(axes, shape, steps):
        _, s, e = om.cuda_bin_edges(nn, d)
        for v in (s, e, np.nextafter(e, np.float32(-1e9)), np.nextafter(s, np.float32(-1e9))):
            p = np.zeros(3, np.float32)
            p[ax] = v
            edge.append(p)
    xyz = np.concatenate([xyz, np.array(edge, np.float32)])
    el = np.concatenate([el, np.full(len(edge), 8)])
    _, xyz_s, uz, cnt = om.sort_elements_and_count(el, xyz, [1, 8, 92])
    ref = om.bin_atoms_cuda(xyz_s, cnt, shape, steps)
    if len(shape) == 2:
        b = eng.OneSliceBuilder(list(uz), shape[0], shape[1], steps[0], steps[1])
        got = _np(b.bin_atoms_one_slice(xyz_s, cnt))
    else:
        b = eng.MultiSlicesBuilder(list(uz), shape[0], shape[1], shape[2], steps[0], steps[1], steps[2])
        got = _np(b.bin_atoms_multi_slices(xyz_s, cnt))
    np.testing.assert_array_equal(got, ref)
    assert got[list(uz).index(92)].sum() == 0


def test_binning_empty(eng):
    b = eng.MultiSlicesBuilder([6], 3, 16, 16, 1.0, 1.0, 1.0)
    got = _np(b.bin_atoms_multi_slices(np.zeros((0, 3), np.float32), np.array([0])))
    assert got.shape == (1, 3, 16, 16) and not got.any()


# ---------------------------------------------------------------------------------
# projected-potential slices
# ---------------------------------------------------------------------------------
@pytest.mark.parametrize("ns,n1,n2", [(1, 64, 64), (3, 64, 64), (4, 128, 256), (5, 256, 256), (2, 48, 48),
                                      (3, 33, 31), (1, 512, 512)])
def test_make_slices(eng, ns, n1, n2):
    rng = np.random.default_rng(ns * 100 + n1)
    zs = [6, 7, 8, 16]
    d = 0.5
    hist = rng.poisson(0.05, size=(len(zs), ns, n1, n2)).astype(np.float32)
    sf = om.scattering_factors_half(zs, n1, n2, d, d)
    for bl in (True, False):
        b = eng.MultiSlicesBuilder(zs, ns, n1, n2, 1.0, d, d)
        got = _np(b.make_multi_slices(hist, symmetric_bandlimit=bl))
        r32 = om.make_slices(hist, sf, "fftw", np.float32, bandlimit=bl)
        r64 = om.make_slices(hist, sf, "fftw", np.float64, bandlimit=bl)
        assert got.shape == (ns, n1, n2)
        assert om.rel_l2(got, r32) < TOL
        assert om.rel_l2(got, r64) < TOL


def test_make_one_slice(eng):
    rng = np.random.default_rng(21)
    zs = [6, 14, 29, 79, 92]
    hist = rng.poisson(0.02, size=(5, 128, 128)).astype(np.float32)
    b = eng.OneSliceBuilder(zs, 128, 128, 0.4, 0.4)
    got = _np(b.make_one_slice(hist))
    ref = om.make_slices(hist, om.scattering_factors_half(zs, 128, 128, 0.4, 0.4), "fftw", np.float64)
    assert om.rel_l2(got, ref) < TOL


# ---------------------------------------------------------------------------------
# end to end
# ---------------------------------------------------------------------------------
def test_five_atoms_512(eng):
    """Five atoms (C, Si, Cu, Au, U) at 512^2, Scherzer, one slice through transmit + lens."""
    from emsim_gb300 import atoms, pot, tem
    el, xyz = om.five_atoms()
    t = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10.37e-3)
    t.set_scherzer_condition()
    pix = 50 / 512
    mol = atoms.AtomList(el, xyz)
    prop = t.get_wave_propagator(wave_shape=(512, 512), pixel_size=pix)
    aslice = pot.build_one_slice(mol, pixel_size=pix, lateral_size=(512, 512))
    ew = prop.slice_transmit(prop.init_wave(), aslice)
    img = _np(eng.intensity(prop.lens_propagate(ew)))
    _, xyz_s, uz, cnt = om.sort_elements_and_count(el, xyz)
    sf = om.scattering_factors_half(list(uz), 512, 512, pix, pix)
    s64 = om.make_slices(om.bin_atoms_cuda(xyz_s, cnt, (512, 512), (pix, pix)), sf, "fftw", np.float64)
    assert om.rel_l2(_np(aslice), s64) < TOL
    w64 = om.WavePropagator(512, 512, pix, pix, 200.0, "fftw", np.float64)
    e64 = w64.slice_transmit(w64.init_wave(20.0), s64)
    i64 = om.intensity(w64.lens_propagate(e64, 1.3, t.defocus, t.aperture))
    assert om.rel_l2(_np(ew), e64) < TOL
    assert om.rel_l2(img, i64) < TOL
    # the image contrast is ~0.4 % of the mean, so float32 intensities alone carry ~1e-3
    # rel-L2 on I - mean; the engine must sit at the FP32 restatement's own level
    w32 = om.WavePropagator(512, 512, pix, pix, 200.0, "fftw", np.float32)
    s32 = om.make_slices(om.bin_atoms_cuda(xyz_s, cnt, (512, 512), (pix, pix)), sf, "fftw", np.float32)
    i32 = om.intensity(w32.lens_propagate(w32.slice_transmit(w32.init_wave(20.0), s32), 1.3, t.defocus, t.aperture))
    floor = om.rel_l2(i32 - i32.mean(), i64 - i64.mean())
    assert om.rel_l2(img - img.mean(), i64 - i64.mean()) < max(2 * floor, 1e-4)


@pytest.mark.parametrize("roi,n_atoms", [(64, 3000), (256, 50000)])
def test_pipe_run(eng, roi, n_atoms):
    from emsim_gb300 import atoms, pipe, tem
    el, xyz = om.protein_blob(n_atoms, radius=40.0 if roi == 256 else 12.0, seed=roi)
    t = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    res = 2.0 if roi == 256 else 1.0
    p = pipe.Pipe(t, resolution=res, slice_thickness=2.0, roi=roi, add_water=False)
    img = _np(p.run(atoms.AtomList(el, xyz)))
    kw = dict(resolution=res, slice_thickness=2.0, roi=roi, beam_energy_kev=200, dose=20, cs_mm=1.3, defocus=700,
              aperture=10e-3, semantics="fftw")
    i32 = om.pipe_run(el, xyz, dtype=np.float32, **kw)
    i64 = om.pipe_run(el, xyz, dtype=np.float64, **kw)
    assert om.rel_l2(img, i32) < TOL
    assert om.rel_l2(img, i64) < TOL
    # the exit wave through the reference-shaped calls
    ew = _np(p.get_exit_wave(atoms.AtomList(el, xyz)))
    _, e64 = om.pipe_run(el, xyz, dtype=np.float64, return_exit_wave=True, **kw)
    assert om.rel_l2(ew, e64) < TOL


def test_fused_image_matches_separate_calls(eng):
    rng = np.random.default_rng(31)
    n, ns = 256, 7
    wp = eng.WavePropagator(n, n, 0.5, 0.5, 200.0)
    sl = (rng.random((2, ns, n, n)) * 2).astype(np.float32)
    dfs = [600.0, 900.0]
    img, ew = wp.image(sl, 2.0, 20.0, 1.3, dfs, 0.011, return_exit_wave=True)
    for b in range(2):
        e = wp.multislice_propagate(wp.init_wave(20.0), sl[b], 2.0)
        i = eng.intensity(wp.lens_propagate(e, 1.3, dfs[b], 0.011))
        assert om.rel_l2(_np(ew)[b], _np(e)) < 1e-6
        assert om.rel_l2(_np(img)[b], _np(i)) < 1e-6


def test_large_wave_properties(eng):
    """2048^2 x 8 slices: a flat potential leaves the plane wave flat (phase only), and
    propagation of a band-limited wave preserves its norm (Parseval)."""
    n = 2048
    wp = eng.WavePropagator(n, n, 0.1, 0.1, 300.0)
    w0 = wp.init_wave(20.0)
    flat = np.full((8, n, n), 0.7, np.float32)
    out = _np(wp.multislice_propagate(w0, flat, 0.5))
    amp = np.sqrt(20.0 * 0.1 * 0.1)
    sig = om.wave_length(300) * om.relativity_gamma(300)
    expect = amp * np.exp(1j * sig * 0.7 * 8)
    assert np.abs(out - expect).max() < 1e-5 * amp
    rng = np.random.default_rng(41)
    w = _rand_wave(rng, (n, n))
    bl = _np(wp.space_propagate(w, 0.0))  # band-limit only (P = 1 at dz = 0)
    p = _np(wp.space_propagate(bl, 7.0))
    assert abs(np.linalg.norm(p) / np.linalg.norm(bl) - 1) < 1e-5


def test_no_device_error_after_runs(eng):
    from emsim_gb300 import _native
    wp = eng.WavePropagator(256, 256, 0.5, 0.5, 200.0)
    sl = np.random.default_rng(51).random((2, 3, 256, 256)).astype(np.float32)
    wp.image(sl, 2.0, 20.0, 1.3, [700.0, 800.0], 0.01)
    assert _native.check_device_error() == 0


def test_tma_and_simple_passes_agree(eng, tmp_path):
    """The persistent TMA-staged passes and the one-tile-per-CTA passes are the same
    arithmetic; run the simple ones in a child process and compare."""
    import subprocess
    import sys
    rng = np.random.default_rng(52)
    sl = (rng.random((2, 4, 512, 512)) * 2).astype(np.float32)
    np.save(tmp_path / "sl.npy", sl)
    code = ("import numpy as np, sys; sys.path.insert(0, %r)\n"
            "from emsim_gb300 import backend\n"
            "wp = backend.WavePropagator(512, 512, 0.5, 0.5, 200.0)\n"
            "sl = np.load(%r)\n"
            "img, ew = wp.image(sl, 2.0, 20.0, 1.3, [700.0, 900.0], 0.01, return_exit_wave=True)\n"
            "np.save(%r, img.get()); np.save(%r, ew.get())\n") % (
        str(__import__("pathlib").Path(__file__).resolve().parent.parent), str(tmp_path / "sl.npy"),
        str(tmp_path / "img.npy"), str(tmp_path / "ew.npy"))
    env = dict(__import__("os").environ, EMSIM_GB300_PASSES="simple")
    subprocess.run([sys.executable, "-c", code], check=True, env=env, timeout=300)
    wp = eng.WavePropagator(512, 512, 0.5, 0.5, 200.0)
    img, ew = wp.image(sl, 2.0, 20.0, 1.3, [700.0, 900.0], 0.01, return_exit_wave=True)
    np.testing.assert_array_equal(_np(img), np.load(tmp_path / "img.npy"))
    np.testing.assert_array_equal(_np(ew), np.load(tmp_path / "ew.npy"))


@pytest.mark.parametrize("n", [1024, 2048])
def test_large_fft_parity(eng, n):
    """Full-size transforms on the 1024 / 2048 fast paths against the oracle."""
    rng = np.random.default_rng(n)
    w = _rand_wave(rng, (n, n))
    sl = (rng.random((2, n, n)) * 2).astype(np.float32)
    wp = eng.WavePropagator(n, n, 0.1, 0.1, 300.0)
    o64 = om.WavePropagator(n, n, 0.1, 0.1, 300.0, "fftw", np.float64)
    assert om.rel_l2(_np(wp.multislice_propagate(w, sl, 0.5)), o64.multislice_propagate(w, sl, 0.5)) < TOL
    assert om.rel_l2(_np(wp.lens_propagate(w, 1.0, 500.0, 0.02)), o64.lens_propagate(w, 1.0, 500.0, 0.02)) < TOL


# ---------------------------------------------------------------------------------
# slices straight from atoms (no histogram)
# ---------------------------------------------------------------------------------
@pytest.mark.parametrize("ns,n", [(40, 256), (7, 64), (1, 128), (16, 512)])
def test_build_slices_from_atoms(eng, ns, n):
    rng = np.random.default_rng(ns * 10 + n)
    zs = [1, 6, 7, 8, 16, 92]
    mols = []
    for k in range(3):
        m = 2000 + 1500 * k
        el = rng.choice(np.array([6, 7, 8, 16, 1]), size=m)  # no uranium: an all-zero element
        half = np.array([ns * 2.0 / 2 * 1.1, n * 0.5 / 2 * 1.1, n * 0.5 / 2 * 1.1])
        xyz = ((rng.random((m, 3)) * 2 - 1) * half).astype(np.float32)
        _, xyz_s, uz, cnt = om.sort_elements_and_count(el, xyz, zs)
        mols.append((xyz_s, cnt))
    b = eng.MultiSlicesBuilder(zs, ns, n, n, 2.0, 0.5, 0.5)
    got = _np(eng.build_slices_batch(b, mols))
    sf = om.scattering_factors_half(zs, n, n, 0.5, 0.5)
    for k, (xyz_s, cnt) in enumerate(mols):
        hist = om.bin_atoms_cuda(xyz_s, cnt, (ns, n, n), (2.0, 0.5, 0.5))
        np.testing.assert_array_equal(_np(b.bin_atoms_multi_slices(xyz_s, cnt)), hist)
        r64 = om.make_slices(hist, sf, "fftw", np.float64)
        r32 = om.make_slices(hist, sf, "fftw", np.float32)
        assert om.rel_l2(got[k], r64) < TOL
        assert om.rel_l2(got[k], r32) < TOL
        dense = _np(b.make_multi_slices(b.bin_atoms_multi_slices(xyz_s, cnt)))
        assert om.rel_l2(got[k], dense) < 1e-6
    # deterministic: a second call is bitwise identical
    np.testing.assert_array_equal(_np(eng.build_slices_batch(b, mols)), got)


def test_build_slices_from_atoms_empty_and_outside(eng):
    b = eng.MultiSlicesBuilder([6, 8], 4, 32, 32, 1.0, 1.0, 1.0)
    far = np.array([[100.0, 0, 0], [0, 100.0, 0]], np.float32)
    got = _np(eng.build_slices_batch(b, [(np.zeros((0, 3), np.float32), [0, 0]), (far, [1, 1])]))
    assert got.shape == (2, 4, 32, 32)
    np.testing.assert_array_equal(got, np.full_like(got, np.float32(1e-13)))


def test_pipe_run_batch_device_front_end(eng):
    """run_batch (GPU centralisation, Z lookup, unsorted atoms) == reference-shaped path
    (host centralize + sort + bin + make) == oracle, for molecules of different element
    sets and sizes, including one that needs a different slice count."""
    from emsim_gb300 import atoms, pipe, tem
    rng = np.random.default_rng(61)
    mols = []
    for k, (n_at, rad, els) in enumerate([(3000, 12.0, (6, 7, 8, 16)), (2500, 12.0, (6, 8)),
                                          (1800, 9.0, (6, 7, 8, 16, 29))]):
        el, xyz = om.protein_blob(n_at, radius=rad, seed=100 + k)
        el = np.asarray(els)[rng.integers(0, len(els), size=n_at)]
        mols.append(atoms.AtomList(el, xyz + rng.normal(size=3).astype(np.float32) * 5))
    t = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    p = pipe.Pipe(t, resolution=1.0, slice_thickness=2.0, roi=64, add_water=False)
    dfs = [650.0, 700.0, 900.0]
    imgs = p.run_batch(mols, defocus=dfs)
    for k, mol in enumerate(mols):
        ref = om.pipe_run(mol.elements, mol.coordinates, resolution=1.0, slice_thickness=2.0, roi=64,
                          beam_energy_kev=200, dose=20, cs_mm=1.3, defocus=dfs[k], aperture=10e-3, semantics="fftw",
                          dtype=np.float64)
        assert om.rel_l2(_np(imgs[k]), ref) < TOL
        # the same image through the per-call reference API shape
        s = p.build_slices(mol)
        wp = p._propagator(s.shape[-2:])
        one = wp.image(s, 2.0, 20.0, 1.3, dfs[k], 10e-3)
        assert om.rel_l2(_np(imgs[k]), _np(one)) < 1e-6
