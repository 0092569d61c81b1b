"""The oracle's native ("fftw") semantics against emsim's own FFTW extension.

tests/golden/make_golden_fftw.py ran the reference's C++ WavePropagator and
MultiSlicesBuilder (compiled from the reference sources against the oracle's FFT
transforms, oracle/ref_fftw) through the reference package's FFTW backend.  The oracle's
FP32 restatement reproduces them to float rounding, its FP64 form to the FP32 error of
the reference's own arithmetic; the numpy backend's semantics (linspace frequency grid)
do not, so the fixture tells the two apart.  Where the reference tree and the built
extension are present the same comparison also runs live on fresh inputs.
"""
import numpy as np
import pytest

from oracle import multislice as om

G = np.load(__import__("pathlib").Path(__file__).parent / "golden" / "golden_fftw_native.npz")
WAVES = sorted({k[1] for k in G.files if k.startswith("w") and k.endswith("_geom")})
SLICES = sorted({k[1] for k in G.files if k.startswith("s") and k.endswith("_geom")})


def _wave_case(tag):
    n1, n2, d, kev, cs, df, ap, dz = G[f"w{tag}_geom"]
    return int(n1), int(n2), float(d), float(kev), float(cs), float(df), float(ap), float(dz)


@pytest.mark.parametrize("tag", WAVES)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_wave_methods_against_reference_fftw(tag, dtype):
    n1, n2, d, kev, cs, df, ap, dz = _wave_case(tag)
    cdt = np.complex64 if dtype == np.float32 else np.complex128
    w = G[f"w{tag}_wave"].astype(cdt)
    s = G[f"w{tag}_slices"].astype(dtype)
    o = om.WavePropagator(n1, n2, d, d, kev, "fftw", dtype)
    assert om.rel_l2(o.slice_transmit(w, s[0]), G[f"w{tag}_transmit"]) < 1e-6
    assert om.rel_l2(o.space_propagate(w, dz), G[f"w{tag}_space"]) < 1e-6
    assert om.rel_l2(o.multislice_propagate(w, s, dz), G[f"w{tag}_multislice"]) < 2e-6
    # the reference evaluates chi in float32: the FP32 restatement follows it to rounding,
    # the FP64 oracle (chi in FP64, as the engine) stays within its float32 phase error
    lens_tol = 1e-6 if dtype == np.float32 else 1e-4
    assert om.rel_l2(o.lens_propagate(w, cs, df, ap), G[f"w{tag}_lens"]) < lens_tol


@pytest.mark.parametrize("tag", WAVES)
def test_numpy_semantics_differ_from_native(tag):
    n1, n2, d, kev, cs, df, ap, dz = _wave_case(tag)
    o = om.WavePropagator(n1, n2, d, d, kev, "numpy", np.float64)
    w = G[f"w{tag}_wave"].astype(np.complex128)
    assert om.rel_l2(o.multislice_propagate(w, G[f"w{tag}_slices"].astype(np.float64), dz),
                     G[f"w{tag}_multislice"]) > 1e-3


@pytest.mark.parametrize("tag", SLICES)
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_slices_against_reference_fftw(tag, dtype):
    ns, n1, n2, d, dz, bl = G[f"s{tag}_geom"]
    n1, n2, d, bl = int(n1), int(n2), float(d), bool(bl)
    zs = [int(z) for z in G[f"s{tag}_zs"]]
    got = om.make_slices(G[f"s{tag}_hist"].astype(dtype), om.scattering_factors_half(zs, n1, n2, d, d), "fftw", dtype,
                         bandlimit=bl)
    assert om.rel_l2(got, G[f"s{tag}_slices"]) < 1e-6


def test_live_reference_fftw_on_fresh_inputs():
    from oracle import ref_numpy
    from oracle.ref_fftw import build as rb
    if not ref_numpy.available() or len(rb.built()) < 2:
        pytest.skip("reference tree or its built FFTW extension not present")
    em = ref_numpy.load_fftw()
    be = em.config.get_current_backend()
    rng = np.random.default_rng(7)
    n1, n2, d, kev = 40, 56, 0.35, 300.0
    wp = be.wave_propagator(n1, n2, d, d, kev)
    w = (rng.normal(size=(n1, n2)) + 1j * rng.normal(size=(n1, n2))).astype(np.complex64)
    s = (rng.random((4, n1, n2)) * 30).astype(np.float32)
    o = om.WavePropagator(n1, n2, d, d, kev, "fftw", np.float32)
    assert om.rel_l2(o.multislice_propagate(w, s, 0.8), wp.multislice_propagate(w, s, 0.8)) < 2e-6
    assert om.rel_l2(o.lens_propagate(w, 1.2, 400.0, 0.015), wp.lens_propagate(w, 1.2, 400.0, 0.015)) < 1e-6
