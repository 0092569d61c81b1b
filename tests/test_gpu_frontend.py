"""The backend calls of emsim's own front-end, replayed through the GB300 backend.

tests/golden/make_frontend_trace.py ran the reference package's front-end with a
recording backend: the five-atom demo chain at 512^2 (pot.build_one_slice,
TEM.get_wave_propagator, init_wave, slice_transmit, lens_propagate) and Pipe.run of a
3000-atom blob at roi 64.  Here every recorded constructor and method call is made on
``emsim_gb300.backend`` with the recorded arguments (numpy inputs, as emsim passes them;
results of earlier calls fed forward), and the final image of each scenario is compared
with

* the same calls replayed through the FP64 oracle (the reference's native FP32
  semantics restated in float64): relative L2 <= 1e-5;
* the reference numpy backend's own output (a stored centre crop): within the numpy
  backend's documented distance from the native semantics (linspace frequency grid,
  numpy binning start edge for odd slice counts), measured on the oracle.
"""
import numpy as np
import pytest

import frontend_trace as ft
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


def test_frontend_trace_replays_through_gb300_backend(eng):
    trace, arrays = ft.load()
    records = trace["records"]
    ours = ft.replay(eng, records, arrays)
    fp64 = ft.replay(ft.oracle_backend("fftw", np.float64), records, arrays)
    numpy_sem = ft.replay(ft.oracle_backend("numpy", np.float64), records, arrays)
    for sc in trace["scenarios"]:
        k = sc["output"]
        out = ours[k]
        assert type(out).__name__ == "DeviceArray" and out.is_cuda
        img = om.intensity(out.get().astype(np.complex128))
        ref = om.intensity(fp64[k])
        err = om.rel_l2(img, ref)
        print(f"\n{sc['name']}: GB300 vs FP64 oracle (native semantics) rel-L2 {err:.3e}")
        assert err < TOL, (sc["name"], err)
        # the reference numpy backend's own output, as far as its semantics allow
        stored = arrays[sc["name"] + "_crop"]
        c = trace["crop"]
        # the oracle's numpy semantics reproduce the stored crop up to the host FFT library's
        # rounding (bit-exact on the machine that recorded it; ~1e-8 on another host)
        assert om.rel_l2(ft.crop(om.intensity(numpy_sem[k]), c), stored) < 1e-6
        delta = om.rel_l2(ft.crop(ref, c), stored)
        got = om.rel_l2(ft.crop(img, c), stored)
        print(f"   vs the reference numpy backend's crop: {got:.3e} (semantic distance {delta:.3e})")
        assert got < 1.01 * delta + 1e-5
