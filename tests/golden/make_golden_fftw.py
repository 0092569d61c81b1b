"""Golden vectors of emsim's native FP32 semantics, made by running the reference's own
FFTW extension (``emsim/backend/fftw_ext/src``: WavePropagator.cpp, SliceBuilder.cpp and
their pybind11 bindings, compiled unchanged by ``oracle/ref_fftw/build.py`` against the
oracle's double-precision transforms in place of libfftw3f) through the reference
package's FFTW backend (``emsim/backend/{wave_propagator,slice_builder}_fftw.py``).

Cases: waves at 64 x 48 (pixel 0.3 A, 200 kV), 64 x 64 (0.5 A, 300 kV) and 33 x 31
(0.25 A, 120 kV): slice_transmit, singleslice_propagate (a zero slice: the free-space
propagation done in place, as multislice does it), multislice_propagate over three
slices, lens_propagate; slices from element histograms at 64^2 (C, O; 4 slices) and
33^2 (C, Au; 5 slices) with the symmetric band-limit, 48 x 40 (H, C, Cu; 3 slices)
without it (the reference's band-limit raises for n1 != n2).  Inputs are stored next to
the outputs.  The reference's standalone ``space_propagate`` is not recorded: for an
out-of-place call it multiplies the input wave, not its spectrum, by the propagator
(WavePropagator.cpp:57-87 reads ``wave`` after transforming into ``waveOut``).

Usage:  python tests/golden/make_golden_fftw.py
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
os.environ.setdefault("EMSIM_REFERENCE_ROOT", "/root/reference")

from oracle import ref_numpy  # noqa: E402

WAVES = {"a": (64, 48, 0.3, 200.0, 1.3, 700.0, 0.02),
         "b": (64, 64, 0.5, 300.0, 1.0, 500.0, 0.01),
         "c": (33, 31, 0.25, 120.0, 2.0, 300.0, 0.03)}
SLICES = {"a": ([6, 8], 4, 64, 64, 0.5, True),
          "b": ([6, 79], 5, 33, 33, 0.25, True),
          "c": ([1, 6, 29], 3, 48, 40, 0.3, False)}
DZ = 1.0


def main():
    em = ref_numpy.load_fftw()
    be = em.config.get_current_backend()
    rng = np.random.default_rng(2024)
    out = {}
    for tag, (n1, n2, d, kev, cs, df, ap) in WAVES.items():
        wp = be.wave_propagator(n1, n2, d, d, kev)
        w = (rng.normal(size=(n1, n2)) + 1j * rng.normal(size=(n1, n2))).astype(np.complex64)
        s = (rng.random((3, n1, n2)) * 20).astype(np.float32)
        out[f"w{tag}_geom"] = np.array([n1, n2, d, kev, cs, df, ap, DZ])
        out[f"w{tag}_wave"] = w
        out[f"w{tag}_slices"] = s
        out[f"w{tag}_transmit"] = wp.slice_transmit(w, s[0])
        out[f"w{tag}_space"] = wp.singleslice_propagate(w, np.zeros((n1, n2), np.float32), DZ)
        out[f"w{tag}_multislice"] = wp.multislice_propagate(w, s, DZ)
        out[f"w{tag}_lens"] = wp.lens_propagate(w, cs, df, ap)
    for tag, (zs, ns, n1, n2, d, bl) in SLICES.items():
        b = be.multi_slices_builder(zs, ns, n1, n2, DZ, d, d)
        hist = ((rng.random((len(zs), ns, n1, n2)) < 0.01) * rng.integers(1, 3, size=(len(zs), ns, n1, n2)))
        hist = hist.astype(np.float32)
        out[f"s{tag}_geom"] = np.array([ns, n1, n2, d, DZ, int(bl)])
        out[f"s{tag}_zs"] = np.array(zs)
        out[f"s{tag}_hist"] = hist
        out[f"s{tag}_slices"] = b.make_multi_slices(hist, symmetric_bandlimit=bl)
    np.savez_compressed(HERE / "golden_fftw_native.npz", **out)
    print(f"{len(out)} arrays, {(HERE / 'golden_fftw_native.npz').stat().st_size} bytes")


if __name__ == "__main__":
    main()
