"""Pin the oracle against golden vectors produced by the reference's own numpy path
(tests/golden/make_golden.py), and check the FFTW/CUDA-semantics restatement for the
documented deltas only."""
import math

import numpy as np
import pytest

from oracle import multislice as om


def test_physics_bit_exact(golden):
    g = golden("physics")
    for f, key in [(om.wave_length, "wave_length"), (om.relativity_gamma, "gamma"),
                   (om.interaction_parameter, "sigma")]:
        np.testing.assert_array_equal(np.array([f(k) for k in g["kev"]]), g[key])
    for kev, cs, df, ap in g["scherzer"]:
        assert om.scherzer(om.wave_length(kev), cs) == (df, ap)


def test_physics_known_answer():
    # emsim/test/physics_test.py:8-16: lambda * gamma == sigma * 2 pi a0 e * 1e8 at 200 keV
    lam, gam, sig = om.wave_length(200), om.relativity_gamma(200), om.interaction_parameter(200)
    assert abs(lam * gam - sig * 2 * math.pi * om.A0_CM * om.E_STATC * 1e8) < 1e-5
    assert abs(lam - 0.025079340612) < 1e-11


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_scattering_factors_bit_exact(golden, tag):
    g = golden("scattering")
    n1, n2, d1, d2 = g[f"grid_{tag}"]
    zs = list(g["zs"])
    np.testing.assert_array_equal(om.scattering_factors2d(zs, int(n1), int(n2), d1, d2), g[f"sf2d_{tag}"])
    np.testing.assert_array_equal(om.scattering_factors_half(zs, int(n1), int(n2), d1, d2), g[f"half_{tag}"])


@pytest.mark.parametrize("tag", ["one_even", "one_odd", "multi_even", "multi_odd"])
def test_numpy_binning_bit_exact(golden, tag):
    g = golden("binning")
    shape = tuple(int(v) for v in g[f"{tag}_shape"])
    steps = tuple(float(v) for v in g[f"{tag}_steps"])
    h = om.bin_atoms_numpy(g[f"{tag}_coords"], g[f"{tag}_counts"], shape, steps)
    np.testing.assert_array_equal(h, g[f"{tag}_hist"])


@pytest.mark.parametrize("tag", ["one_even", "multi_even"])
def test_cuda_rule_matches_numpy_rule_off_edges(golden, tag):
    """For even sizes both rules share the start edge; they differ only for atoms exactly on
    an edge (the numpy rule's float arange edges vs the CUDA rule's right-closed test)."""
    g = golden("binning")
    shape = tuple(int(v) for v in g[f"{tag}_shape"])
    steps = tuple(float(v) for v in g[f"{tag}_steps"])
    xyz = g[f"{tag}_coords"]
    cols = (1, 2) if len(shape) == 2 else (0, 1, 2)
    frac = [(xyz[:, c] / d) % 1.0 for c, d in zip(cols, steps)]
    away = np.all([np.minimum(f, 1 - f) > 1e-3 for f in frac], axis=0)
    inside = np.all([np.abs(xyz[:, c]) < n * d / 2 - 1e-3 for c, n, d in zip(cols, shape, steps)], axis=0)
    keep = away & inside
    el = g[f"{tag}_elements"][keep]
    _, xyz2, uz, cnt = om.sort_elements_and_count(el, xyz[keep])
    a = om.bin_atoms_cuda(xyz2, cnt, shape, steps)
    b = om.bin_atoms_numpy(xyz2, cnt, shape, steps)
    # float arange edges can add one bin past the end (dz = 1.3 here); compare the box
    b = b[(slice(None),) + tuple(slice(0, n) for n in shape)]
    assert a.sum() == len(el)
    np.testing.assert_array_equal(a, b)


def test_cuda_rule_edges_and_outside():
    # n = 4, d = 1: CUDA rule start = -d*floor(5/2) = -2, end = 2; [start, end] closed
    xyz = np.array([[0, -2.0, 0], [0, 2.0, 0], [0, 1.999999, 0], [0, -2.000001, 0], [0, 2.000001, 0],
                    [0, 0.0, 0]], np.float32)
    h = om.bin_atoms_cuda(xyz, np.array([6]), (4, 4), (1.0, 1.0))
    assert h.sum() == 4  # two outside atoms dropped
    assert h[0, 0, 2] == 1 and h[0, 3, 2] == 2 and h[0, 2, 2] == 1
    # odd n: start = -d * floor((n+1)/2) = -3 for n = 5 (numpy rule: -d * (n//2) = -2)
    d32, start, end = om.cuda_bin_edges(5, 1.0)
    assert start == -3.0 and end == 2.0
    assert om.numpy_bin_edges(5, 1.0)[0] == -2.0


def test_make_slices_numpy_bit_exact(golden):
    g = golden("slices")
    np.testing.assert_array_equal(om.make_slices(g["ms_hist"], g["ms_sf"], "numpy"), g["ms_slices"])
    np.testing.assert_array_equal(om.make_slices(g["os_hist"], g["ms_sf"], "numpy"), g["os_slice"])


def test_make_slices_fftw_vs_numpy(golden):
    """Same math, different precision: FFTW semantics in FP64 equals the numpy path (which
    runs its first stage in float32) to float32 accuracy."""
    g = golden("slices")
    v64 = om.make_slices(g["ms_hist"], g["ms_sf"], "fftw", np.float64)
    v32 = om.make_slices(g["ms_hist"], g["ms_sf"], "fftw", np.float32)
    assert om.rel_l2(v64, g["ms_slices"]) < 1e-6
    assert om.rel_l2(v32, v64) < 1e-6


def test_front_end_slices_bit_exact(golden):
    g = golden("slices")
    el, xyz = g["five_elements"], g["five_coords"]
    _, xyz_s, uz, cnt = om.sort_elements_and_count(el, xyz)
    h = om.bin_atoms_numpy(xyz_s, cnt, (48, 48), (50 / 48, 50 / 48))
    sf = om.scattering_factors_half(list(uz), 48, 48, 50 / 48, 50 / 48)
    np.testing.assert_array_equal(om.make_slices(h, sf, "numpy"), g["five_slice"])
    blob = om.build_multi_slices(g["blob_elements"], g["blob_coords"], 2.0, 1.0, 16, None, "numpy")
    np.testing.assert_array_equal(blob, g["blob_slices"])


@pytest.mark.parametrize("tag", ["sq", "rect"])
def test_wave_numpy_bit_exact(golden, tag):
    g = golden("wave")
    n1, n2, d = g[f"{tag}_grid"]
    wp = om.WavePropagator(int(n1), int(n2), d, d, 200.0, "numpy")
    x, sl = g[f"{tag}_wave"], g[f"{tag}_slices"]
    cs, df, ap = g[f"{tag}_lens_params"]
    np.testing.assert_array_equal(wp.init_wave(20.0), g[f"{tag}_init"])
    np.testing.assert_array_equal(wp.slice_transmit(x, sl[0]), g[f"{tag}_transmit"])
    np.testing.assert_array_equal(wp.space_propagate(x, 2.0), g[f"{tag}_space"])
    np.testing.assert_array_equal(wp.singleslice_propagate(x, sl[0], 2.0), g[f"{tag}_single"])
    np.testing.assert_array_equal(wp.multislice_propagate(x, sl, 2.0), g[f"{tag}_multi"])
    np.testing.assert_array_equal(wp.lens_propagate(x, cs, df, ap), g[f"{tag}_lens"])


def test_pipe_numpy_bit_exact(golden):
    g = golden("pipe")
    img = om.pipe_run(g["blob_elements"], g["blob_coords"], resolution=2.0, slice_thickness=2.0, roi=32,
                      beam_energy_kev=200, dose=20, cs_mm=1.3, defocus=700, aperture=10e-3, semantics="numpy")
    np.testing.assert_array_equal(img, g["blob_image"])


def test_five_atoms_numpy_and_fftw(golden):
    g = golden("pipe")
    df, ap = g["five_tem"]
    el, xyz = om.five_atoms()
    _, xyz_s, uz, cnt = om.sort_elements_and_count(el, xyz)
    pix = 50 / 128
    sf = om.scattering_factors_half(list(uz), 128, 128, pix, pix)
    s_np = om.make_slices(om.bin_atoms_numpy(xyz_s, cnt, (128, 128), (pix, pix)), sf, "numpy")
    np.testing.assert_array_equal(s_np, g["five_slice"])
    wp = om.WavePropagator(128, 128, pix, pix, 200.0, "numpy")
    ew = wp.slice_transmit(wp.init_wave(20.0), s_np)
    np.testing.assert_array_equal(ew, g["five_exit"])
    np.testing.assert_array_equal(np.abs(wp.lens_propagate(ew, 1.3, df, ap)) ** 2, g["five_image"])
    # FFTW semantics (fftfreq grid, f^2 <= aperture^2): close to the numpy image, not equal
    s_f = om.make_slices(om.bin_atoms_cuda(xyz_s, cnt, (128, 128), (pix, pix)), sf, "fftw", np.float64)
    wf = om.WavePropagator(128, 128, pix, pix, 200.0, "fftw", np.float64)
    img_f = om.intensity(wf.lens_propagate(wf.slice_transmit(wf.init_wave(20.0), s_f), 1.3, df, ap))
    assert om.rel_l2(img_f, g["five_image"]) < 1e-3


def test_fftw_fp32_vs_fp64():
    el, xyz = om.protein_blob(3000, radius=12.0, seed=3)
    kw = dict(resolution=1.0, slice_thickness=2.0, roi=64, beam_energy_kev=200, dose=20, cs_mm=1.3, defocus=700,
              aperture=10e-3, semantics="fftw")
    i32, e32 = om.pipe_run(el, xyz, dtype=np.float32, return_exit_wave=True, **kw)
    i64, e64 = om.pipe_run(el, xyz, dtype=np.float64, return_exit_wave=True, **kw)
    assert om.rel_l2(e32, e64) < 1e-5
    assert om.rel_l2(i32, i64) < 1e-5


def test_freq_grid_is_fftfreq():
    for n1, n2, d1, d2 in [(8, 8, 0.5, 0.5), (7, 10, 0.3, 0.4)]:
        f2 = om.fftw_freq_sq(n1, n2, d1, d2, np.float64)
        fx = np.fft.fftfreq(n1, d1)
        fy = np.fft.fftfreq(n2, d2)
        np.testing.assert_allclose(f2, fx[:, None] ** 2 + fy[None, :] ** 2, rtol=1e-14)


def test_band_limit_specimen_golden():
    """oracle.band_limit_slices against the reference's band_limit_specimen, run on a
    cubic stack (axes (0, 1) of the reference = the lateral axes of the transposed stack)."""
    from pathlib import Path
    g = np.load(Path(__file__).resolve().parent / "golden" / "golden_specimen.npz")
    cube = g["cube"]
    got = om.band_limit_slices(np.moveaxis(cube, 2, 0))
    np.testing.assert_allclose(np.moveaxis(got, 0, 2), g["band_limited"], rtol=1e-12, atol=1e-12)
