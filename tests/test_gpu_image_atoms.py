"""Image formation straight from atoms with the slices built chunk by chunk
(emsim_gb300_image_from_atoms_z): bitwise equal to the slice build followed by the fused
image for every chunk size, including an odd slice count (a half-empty last pair) and a
chunk size that does not divide the pair count, with the per-tile (128^2, 256^2) and the
persistent (512^2) slice column pass; and the Pipe route that uses it for
large stacks against the FP64 oracle.
"""
import numpy as np
import pytest

from oracle import multislice as om

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import torch  # noqa: F401

    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import backend
    return backend


def _device_batch(backend, mols):
    import torch
    dev = torch.device("cuda", torch.cuda.current_device())
    offsets = np.zeros(len(mols) + 1, dtype=np.int64)
    offsets[1:] = np.cumsum([len(el) for el, _ in mols])
    xyz = torch.from_numpy(np.concatenate([x for _, x in mols]).astype(np.float32)).to(dev)
    z = torch.from_numpy(np.concatenate([el for el, _ in mols]).astype(np.int32)).to(dev)
    off = torch.from_numpy(offsets.astype(np.uint32).view(np.int32)).to(dev)
    nm = len(mols)
    shift = torch.empty((nm, 3), dtype=torch.float32, device=dev)
    space = torch.empty((nm, 3), dtype=torch.float32, device=dev)
    P = backend._ptr
    backend._native.call("emsim_gb300_centralize", P(xyz), P(z), P(off), nm, P(shift), P(space), None,
                         backend._stream())
    return xyz, z, off, shift


@pytest.mark.parametrize("n,ns", [(128, 9), (256, 12), (512, 7)])
def test_chunked_image_bitwise_equal(eng, n, ns):
    backend = eng
    mols = [om.protein_blob(3000 + 500 * k, radius=18.0, seed=40 + k) for k in range(3)]
    xyz, z, off, shift = _device_batch(backend, mols)
    zs = [6, 7, 8, 16]
    b = backend.MultiSlicesBuilder(zs, ns, n, n, 2.0, 0.5, 0.5)
    wp = backend.WavePropagator(n, n, 0.5, 0.5, 200.0)
    dfs = [600.0, 700.0, 800.0]
    idx = [0, 1, 2]
    stack = backend.build_slices_from_device_atoms(b, xyz, z, off, shift, idx, 3)
    ref = wp.image(stack, 2.0, 20.0, 1.3, dfs, 10e-3).get()
    for chunk in (1, 2, 4, 0):
        got = backend.image_from_device_atoms(b, wp, xyz, z, off, shift, idx, 3, 20.0, 1.3, dfs, 10e-3,
                                              chunk_pairs=chunk).get()
        np.testing.assert_array_equal(got, ref, err_msg=f"chunk {chunk}")


def test_pipe_large_stack_route_against_fp64(eng, monkeypatch):
    """Pipe.run_batch builds stacks above its size limit chunk by chunk; lowered here so a
    small molecule takes that route."""
    from emsim_gb300 import atoms, pipe, tem
    monkeypatch.setattr(pipe, "_STACK_LIMIT_BYTES", 1 << 20)
    el, xyz = om.protein_blob(4000, radius=16.0, seed=9)
    t = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    p = pipe.Pipe(t, resolution=1.0, slice_thickness=2.0, roi=128, add_water=False)
    img = p.run_batch([atoms.AtomList(el, xyz)], to_host=True)[0]
    ref = om.pipe_run(el, xyz, resolution=1.0, slice_thickness=2.0, roi=128, beam_energy_kev=200, dose=20,
                      cs_mm=1.3, defocus=700, aperture=10e-3, semantics="fftw", dtype=np.float64)
    assert om.rel_l2(img, ref) < 1e-5
