"""Specimen band-limit (tem.band_limit_specimen), the weak-phase pipeline (Pipe.run_wpo)
and the pipeline with voxel water on the GPU."""
import numpy as np
import pytest

from oracle import multislice as om

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import atoms, pipe, tem
    return atoms, pipe, tem


@pytest.mark.parametrize("shape", [(5, 64, 64), (4, 128, 32), (1, 256, 256), (3, 16, 64)])
def test_band_limit_specimen(eng, shape):
    _, _, tem = eng
    x = (np.random.default_rng(sum(shape)).random(shape) * 10).astype(np.float32)
    got = np.asarray(tem.band_limit_specimen(tem.Specimen(x, 1.0, 2.0)).slices.get())
    ref = om.band_limit_slices(x)
    assert got.shape == x.shape
    assert om.rel_l2(got, ref) < 1e-6


def test_run_wpo_matches_oracle(eng):
    atoms, pipe, tem = eng
    el, xyz = om.five_atoms()
    t = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    t.set_scherzer_condition()
    p = pipe.Pipe(t, resolution=2 * 50 / 512, slice_thickness=1.0, roi=512, add_water=False)
    got = np.asarray(p.run_wpo(atoms.AtomList(el, xyz)).get())
    wp = om.WavePropagator(512, 512, 50 / 512, 50 / 512, 200.0, "fftw", np.float64)
    c = om.centralize(xyz)
    _, cs, uz, cnt = om.sort_elements_and_count(np.asarray(el), c)
    hist = om.bin_atoms_cuda(cs, cnt, (512, 512), (50 / 512, 50 / 512))
    sf = om.scattering_factors_half(list(uz), 512, 512, 50 / 512, 50 / 512)
    aslice = om.make_slices(hist, sf, "fftw", np.float64)
    ew = wp.singleslice_propagate(wp.init_wave(20.0), aslice, 0.0)
    ref = om.intensity(wp.lens_propagate(ew, 1.3, t.defocus, t.aperture))
    assert om.rel_l2(got, ref) < 1e-5


def test_pipe_with_water(eng):
    atoms, pipe, tem = eng
    el, xyz = om.protein_blob(3000, radius=12.0, seed=3)
    el = np.where(np.arange(len(el)) % 7 == 0, 1, el)  # some hydrogens: Z = 1 and 8 present
    t = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    p = pipe.Pipe(t, resolution=2.0, slice_thickness=2.0, roi=64, add_water=True)
    mol = atoms.AtomList(el, xyz)
    np.random.seed(5)
    a = np.asarray(p.run(mol).get())
    np.random.seed(5)
    b = np.asarray(p.run(mol).get())
    np.testing.assert_array_equal(a, b)  # the water seed comes from numpy's global generator
    dry = np.asarray(pipe.Pipe(t, resolution=2.0, slice_thickness=2.0, roi=64, add_water=False).run(mol).get())
    assert np.isfinite(a).all() and not np.allclose(a, dry)
