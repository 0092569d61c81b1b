"""Failure detection on the GPU without a fault: a bounded mbarrier wait that runs out.

emsim_gb300_wait_timeout_probe launches one CTA that waits, bounded, on an mbarrier
nothing arrives at (no copy is in flight), exactly the wait the TMA-pipelined passes use
for their tile copies.  The test checks that the kernel returns, that the timeout lands in
the device error word (mapped host memory, readable without a device synchronisation),
that the Python API raises on it at its host sync points, that emsim_gb300_check_device_error
reads and clears it, and that the context stays usable afterwards.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import torch  # noqa: F401

    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import _native, backend
    return _native, backend


def _probe(nat, backend, limit_ns):
    import torch
    done = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    nat.call("emsim_gb300_wait_timeout_probe", int(limit_ns), backend._ptr(done), backend._stream())
    torch.cuda.synchronize()
    return int(done.item())


def test_bounded_wait_times_out_and_is_reported(eng):
    import time

    nat, backend = eng
    assert nat.check_device_error() == 0
    t0 = time.perf_counter()
    assert _probe(nat, backend, 5_000_000) == 0  # 5 ms: the wait gave up
    assert time.perf_counter() - t0 < 5.0
    assert nat.peek_device_error() == 1
    with pytest.raises(nat.DeviceWaitTimeout):
        nat.raise_on_device_error()
    assert nat.check_device_error() == 1  # read and cleared
    assert nat.peek_device_error() == 0
    assert nat.check_device_error() == 0


def test_api_raises_after_a_timeout_and_context_stays_usable(eng):
    from emsim_gb300 import atoms, pipe, tem
    from oracle import multislice as om

    nat, backend = eng
    el, xyz = om.protein_blob(800, radius=8.0, seed=3)
    p = pipe.Pipe(tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3),
                  resolution=1.0, slice_thickness=2.0, roi=32, add_water=False)
    mol = atoms.AtomList(el, xyz)
    good = p.run_batch([mol], to_host=True)[0]
    assert _probe(nat, backend, 2_000_000) == 0
    with pytest.raises(nat.DeviceWaitTimeout):
        p.run_batch([mol], to_host=True)
    with pytest.raises(nat.DeviceWaitTimeout):
        p.run(mol).get()
    assert nat.check_device_error() == 1
    again = p.run_batch([mol], to_host=True)[0]
    assert np.array_equal(good, again)
    assert nat.check_device_error() == 0


def test_wait_limit_reaches_the_pipelined_kernels(eng):
    """A shorter (but ample) limit leaves the pipelined passes' results unchanged."""
    import torch

    nat, backend = eng
    rng = np.random.default_rng(5)
    w = (rng.normal(size=(4, 256, 256)) + 1j * rng.normal(size=(4, 256, 256))).astype(np.complex64)
    sl = rng.random((4, 3, 256, 256)).astype(np.float32)
    wp = backend.WavePropagator(256, 256, 0.5, 0.5, 200.0)
    ref = wp.multislice_propagate(w, sl, 2.0).get()
    lib = nat.load()
    old = lib.emsim_gb300_get_wait_limit_ns()
    try:
        assert lib.emsim_gb300_set_wait_limit_ns(100_000_000) == 0
        out = wp.multislice_propagate(w, sl, 2.0).get()
    finally:
        lib.emsim_gb300_set_wait_limit_ns(old)
    torch.cuda.synchronize()
    assert np.array_equal(ref, out)
    assert nat.check_device_error() == 0
