"""The engine against emsim's own native implementation: golden outputs of the
reference's FFTW extension (WavePropagator.cpp / SliceBuilder.cpp run through the
reference package's FFTW backend, tests/golden/make_golden_fftw.py) on the same inputs.

Waves at 64 x 48, 64^2 and 33 x 31 (odd sizes take the generic-length path): transmit,
in-place free-space propagation, three-slice multislice (rel-L2 <= 1e-5) and the lens,
where the engine evaluates the aberration phase in FP64 and the reference in float32
(rel-L2 <= 1e-4, the reference's own phase rounding); slices from element histograms
with and without the symmetric band-limit (rel-L2 <= 1e-5).
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import multislice as om

pytestmark = pytest.mark.gpu

G = np.load(Path(__file__).parent / "golden" / "golden_fftw_native.npz")
WAVES = sorted({k[1] for k in G.files if k.startswith("w") and k.endswith("_geom")})
SLICES = sorted({k[1] for k in G.files if k.startswith("s") and k.endswith("_geom")})


@pytest.fixture(scope="module")
def backend():
    import torch  # noqa: F401

    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import backend
    return backend


@pytest.mark.parametrize("tag", WAVES)
def test_wave_methods_against_reference_native(backend, tag):
    n1, n2, d, kev, cs, df, ap, dz = G[f"w{tag}_geom"]
    n1, n2 = int(n1), int(n2)
    wp = backend.WavePropagator(n1, n2, float(d), float(d), float(kev))
    w, s = G[f"w{tag}_wave"], G[f"w{tag}_slices"]
    zero = np.zeros((n1, n2), np.float32)
    assert om.rel_l2(wp.slice_transmit(w, s[0]).get(), G[f"w{tag}_transmit"]) < 1e-5
    assert om.rel_l2(wp.singleslice_propagate(w, zero, float(dz)).get(), G[f"w{tag}_space"]) < 1e-5
    assert om.rel_l2(wp.space_propagate(w, float(dz)).get(), G[f"w{tag}_space"]) < 1e-5
    assert om.rel_l2(wp.multislice_propagate(w, s, float(dz)).get(), G[f"w{tag}_multislice"]) < 1e-5
    assert om.rel_l2(wp.lens_propagate(w, float(cs), float(df), float(ap)).get(), G[f"w{tag}_lens"]) < 1e-4


@pytest.mark.parametrize("tag", SLICES)
def test_slices_against_reference_native(backend, tag):
    ns, n1, n2, d, dz, bl = G[f"s{tag}_geom"]
    zs = [int(z) for z in G[f"s{tag}_zs"]]
    b = backend.MultiSlicesBuilder(zs, int(ns), int(n1), int(n2), float(dz), float(d), float(d))
    got = b.make_multi_slices(G[f"s{tag}_hist"], symmetric_bandlimit=bool(bl)).get()
    assert om.rel_l2(got, G[f"s{tag}_slices"]) < 1e-5
