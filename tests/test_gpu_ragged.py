"""Ragged batches: molecules of one lateral size with different slice counts in one
slice-build call and one image call, and lateral sizes on separate streams; each result
equals the one the molecule gets alone (bitwise) and the FP64 oracle (rel-L2 1e-5)."""
import numpy as np
import pytest

from oracle import multislice as om

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import emsim_gb300.build as b
    b.build()
    import torch

    from emsim_gb300 import atoms, backend, pipe, tem
    return torch, atoms, backend, pipe, tem


def _mols(rng, specs):
    mols = []
    for n_at, rz, rxy in specs:
        el = rng.choice(np.array([6, 7, 8, 16]), size=n_at, p=[0.63, 0.17, 0.19, 0.01])
        xyz = np.column_stack([(rng.random(n_at) * 2 - 1) * rz, (rng.random((n_at, 2)) * 2 - 1) * rxy])
        mols.append((el, xyz.astype(np.float32)))
    return mols


def test_ragged_build_and_image_equal_single(eng):
    torch, atoms, backend, pipe, tem = eng
    rng = np.random.default_rng(3)
    specs = [(2500, 9.0, 20.0), (1800, 21.0, 20.0), (900, 3.0, 20.0), (2000, 15.0, 20.0)]
    mols = [atoms.AtomList(el, xyz) for el, xyz in _mols(rng, specs)]
    t = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    p = pipe.Pipe(t, resolution=1.0, slice_thickness=2.0, roi=64, add_water=False)
    dfs = [600.0, 700.0, 800.0, 900.0]
    imgs = p.run_batch(mols, defocus=dfs)
    ns = []
    for k, mol in enumerate(mols):
        s = p.build_slices(mol)
        ns.append(s.shape[0])
        wp = p._propagator(s.shape[-2:])
        one = np.asarray(wp.image(s, 2.0, 20.0, 1.3, dfs[k], 10e-3).get())
        np.testing.assert_array_equal(np.asarray(imgs[k].get()), one)
        ref = om.pipe_run(mol.elements, mol.coordinates, resolution=1.0, slice_thickness=2.0, roi=64,
                          beam_energy_kev=200, dose=20, cs_mm=1.3, defocus=dfs[k], aperture=10e-3, semantics="fftw",
                          dtype=np.float64)
        assert om.rel_l2(np.asarray(imgs[k].get()), ref) < 1e-5
    assert len(set(ns)) >= 3  # a ragged batch indeed


def test_ragged_slices_equal_per_molecule_stacks(eng):
    torch, atoms, backend, pipe, tem = eng
    rng = np.random.default_rng(4)
    zs = [6, 7, 8, 16]
    specs = [(1500, 11.0, 14.0), (1500, 5.0, 14.0), (1200, 8.0, 14.0)]
    raw = _mols(rng, specs)
    n, dz, d = 64, 2.0, 0.5
    counts = []
    for el, xyz in raw:
        c = om.centralize(xyz)
        space = c.max(axis=0) - c.min(axis=0)
        counts.append(om.finalize_slice_size(space, (d, d), dz, (n, n), None)[0])
    order = np.argsort(-np.array(counts), kind="stable")
    smax = max(counts)
    xyz_all = np.concatenate([xyz for _, xyz in raw]).astype(np.float32)
    z_all = np.concatenate([el for el, _ in raw]).astype(np.int32)
    off = np.concatenate([[0], np.cumsum([len(el) for el, _ in raw])]).astype(np.uint32)
    dev = "cuda"
    X = torch.tensor(xyz_all, device=dev)
    Z = torch.tensor(z_all, device=dev)
    O = torch.tensor(off.view(np.int32), device=dev)
    nm = len(raw)
    shift = torch.empty((nm, 3), dtype=torch.float32, device=dev)
    space = torch.empty((nm, 3), dtype=torch.float32, device=dev)
    P = backend._ptr
    backend._native.call("emsim_gb300_centralize", P(X), P(Z), P(O), nm, P(shift), P(space), None, backend._stream())
    b = backend.MultiSlicesBuilder(zs, smax, n, n, dz, d, d)
    idx = [int(i) for i in order]
    ss = [counts[i] for i in idx]
    stack = np.asarray(backend.build_slices_from_device_atoms(b, X, Z, O, shift, idx, nm, slot_slices=ss).get())
    for j, i in enumerate(idx):
        bi = backend.MultiSlicesBuilder(zs, counts[i], n, n, dz, d, d)
        alone = np.asarray(backend.build_slices_from_device_atoms(bi, X, Z, O, shift, [i], nm).get())[0]
        np.testing.assert_array_equal(stack[j, :counts[i]], alone)


def test_mixed_lateral_sizes_on_streams(eng):
    torch, atoms, backend, pipe, tem = eng
    rng = np.random.default_rng(5)
    specs = [(1500, 8.0, 14.0), (1500, 8.0, 30.0), (1000, 12.0, 14.0), (1200, 6.0, 28.0)]
    mols = [atoms.AtomList(el, xyz) for el, xyz in _mols(rng, specs)]
    t = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    p = pipe.Pipe(t, resolution=2.0, slice_thickness=2.0, roi=None, add_water=False)
    imgs = p.run_batch(mols, to_host=True)
    shapes = {im.shape for im in imgs}
    assert len(shapes) >= 2
    for k, mol in enumerate(mols):
        alone = np.asarray(p.run_batch([mol])[0].get())
        np.testing.assert_array_equal(imgs[k], alone)


def test_large_batch_runs_in_chunks_equal_single(eng):
    """128 molecules of 35k atoms (4.5 M atoms) run as two chunks on two streams; every
    image equals the one its molecule gets alone, bitwise."""
    torch, atoms, backend, pipe, tem = eng
    from emsim_gb300 import synth
    m = tem.TEM(electron_dose=20.0, beam_energy_kev=200.0, cs_mm=1.3, defocus=700.0, aperture=10e-3)
    p = pipe.Pipe(m, resolution=2.0, slice_thickness=2.0, roi=128, add_water=False)
    mols = [atoms.AtomList(*synth.protein_blob(35_000, 30.0 + (i % 5), 500 + i)) for i in range(128)]
    dfs = [600.0 + 5 * i for i in range(128)]
    got = p.run_batch(mols, defocus=dfs, to_host=True)
    for i in (0, 63, 64, 127):
        one = p.run_batch([mols[i]], defocus=[dfs[i]], to_host=True)[0]
        np.testing.assert_array_equal(got[i], one)


def test_submitted_batches_in_flight_equal_serial(eng):
    """Pipe.submit_batch keeps two batches in flight on alternating stream sets (one of
    them chunked, one with two lateral sizes); each PendingImages.result() equals
    run_batch(to_host=True) of the same batch, bitwise and in input order, whatever the
    order the results are collected in."""
    torch, atoms, backend, pipe, tem = eng
    from emsim_gb300 import synth
    m = tem.TEM(electron_dose=20.0, beam_energy_kev=200.0, cs_mm=1.3, defocus=700.0, aperture=10e-3)
    p = pipe.Pipe(m, resolution=2.0, slice_thickness=2.0, roi=128, add_water=False)
    big = [atoms.AtomList(*synth.protein_blob(35_000, 30.0 + (i % 5), 900 + i)) for i in range(128)]
    rng = np.random.default_rng(11)
    small = [atoms.AtomList(el, xyz) for el, xyz in _mols(rng, [(1500, 8.0, 14.0), (1500, 8.0, 30.0),
                                                                 (1000, 12.0, 14.0)])]
    rois = [64, 128, 64]
    batches = [(big, None), (small, rois), (big[::-1], None), (small[::-1], rois[::-1])]
    serial = [p.run_batch(mols, to_host=True, rois=r) for mols, r in batches]
    pend = [p.submit_batch(mols, rois=r) for mols, r in batches[:2]]
    got = [None] * 4
    got[1] = pend[1].result()
    pend.append(p.submit_batch(batches[2][0]))
    got[0] = pend[0].result()
    pend.append(p.submit_batch(batches[3][0], rois=batches[3][1]))
    got[3] = pend[3].result()
    got[2] = pend[2].result()
    assert pend[2].done()
    for g, s in zip(got, serial):
        assert len(g) == len(s)
        for a, b in zip(g, s):
            assert isinstance(a, np.ndarray)
            np.testing.assert_array_equal(a, b)


def test_emsim_batched_equals_run_batch(eng):
    """simulator.EMSim with batch_size 2 (groups through Pipe.submit_batch, two in
    flight) hands each molecule's image to the handler, bitwise equal to run_batch."""
    torch, atoms, backend, pipe, tem = eng
    from emsim_gb300.simulator import EMSim
    rng = np.random.default_rng(21)
    specs = [(1200, 8.0, 14.0), (900, 6.0, 14.0), (1500, 10.0, 14.0), (700, 5.0, 14.0), (1100, 7.0, 14.0)]
    mols = [atoms.AtomList(el, xyz, label=f"mol{i}") for i, (el, xyz) in enumerate(_mols(rng, specs))]
    m = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    p = pipe.Pipe(m, resolution=2.0, slice_thickness=2.0, roi=64, add_water=False)
    ref = p.run_batch(mols, to_host=True)
    got = {}
    EMSim(p, mols, lambda img, label: got.__setitem__(label, np.array(img)), batch_size=2).run()
    assert sorted(got) == [f"mol{i}" for i in range(len(mols))]
    for i in range(len(mols)):
        np.testing.assert_array_equal(got[f"mol{i}"], ref[i])
