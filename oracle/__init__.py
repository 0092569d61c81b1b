"""CPU oracle for emsim's multislice hot path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
CPU-baseline / reference legs of ``bench.py`` import this package, and there only as
the checker or as the timed CPU baseline.  The product package ``emsim_gb300`` never
imports it and never falls back to it.

Contents
--------
``oracle.multislice``  numpy restatement of the reference's algorithm for the path
    atoms -> bins -> projected-potential slices -> multislice -> lens -> intensity,
    in two semantics:

    * ``"fftw"``  - the reference's FP32 native semantics (FFTW C++ extension
      ``emsim/backend/fftw_ext/src/*.cpp`` and CUDA extension
      ``emsim/backend/cuda_ext/src/*.cu``): true fftfreq grid, 2/3 band-limit in every
      propagation, ``f^2 <= (alpha/lambda)^2`` aperture, CUDA binning rule.
      Run with ``dtype=float32`` it is the FP32 restatement; with ``dtype=float64`` it
      is the FP64 oracle.
    * ``"numpy"`` - the reference's numpy backend (``emsim/backend/*_numpy.py`` and
      ``slice_builder_base.py``): ``linspace`` q-grid, numpy histogram binning rule,
      strict aperture, complex128 arithmetic.

``oracle.ref_numpy``  imports the reference's own numpy path, or its FFTW backend with
    the extension that ``oracle.ref_fftw`` builds (only where the reference tree exists,
    i.e. never on a GPU host) to generate golden vectors.

``oracle.ref_fftw``  builds emsim's FFTW extension from the reference C++ sources into
    ``oracle/_ref``, against the oracle's own FFTW-interface transforms (``fftw3.h``,
    ``fftw_stub.cpp``) in place of the absent libfftw3f.

Parity status: PINNED.  ``tests/golden/make_golden.py`` ran the reference's own numpy
path on seeded small inputs; ``tests/test_oracle_golden.py`` checks the ``"numpy"``
semantics against those vectors (bit-exact for binning, ~1e-12 for floating point).
The ``"fftw"`` semantics shares every helper with the pinned path and differs only by
the documented reference deltas (frequency grid, filter placement, aperture test,
binning start edge), each tested separately, and is PINNED too:
``tests/golden/make_golden_fftw.py`` ran the reference's FFTW extension (compiled from
its C++) through its FFTW backend, and ``tests/test_oracle_ref_fftw.py`` checks the FP32
restatement against those vectors to float rounding.
"""
