"""Pipe.run_batch / submit_batch with cuda_graphs=True: a batch structure seen before is
replayed from one CUDA graph of its slice builds and image formation; the images are
bitwise those of the eager launches, for a plain group, a ragged group (molecules of
different slice counts), two lateral sizes, per-molecule defocus values and the chunked
route for large stacks; the copies handed out are not overwritten by later replays."""
import numpy as np
import pytest

from oracle import multislice as om

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mods():
    import torch  # noqa: F401

    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import atoms, pipe, tem
    return atoms, pipe, tem


def _pipes(mods, **kw):
    atoms, pipe, tem = mods
    t = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    args = dict(resolution=1.0, slice_thickness=2.0, roi=128, add_water=False)
    args.update(kw)
    return pipe.Pipe(t, **args), pipe.Pipe(t, cuda_graphs=True, **args)


def _mols(mods, radii, n0=3000):
    atoms = mods[0]
    return [atoms.AtomList(*om.protein_blob(n0 + 400 * k, radius=r, seed=60 + k)) for k, r in enumerate(radii)]


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b)) and len(a) == len(b)


def test_replay_bitwise_equal_to_eager(mods):
    eager, graphed = _pipes(mods)
    mols = _mols(mods, [16.0, 16.0, 16.0])
    ref = eager.run_batch(mols, to_host=True)
    for rep in range(6):
        assert _same(graphed.run_batch(mols, to_host=True), ref), rep
    # to_host batches alternate between two buffer sets (two batches in flight): one graph each
    assert len(graphed._graphs) == 2
    # device results are copies: a later replay leaves them as they were
    first = graphed.run_batch(mols)
    kept = [x.get().copy() for x in first]
    graphed.run_batch(_mols(mods, [15.0, 15.0, 15.0]))
    graphed.run_batch(mols)
    assert _same([x.get() for x in first], kept)
    assert _same(kept, ref)


def test_ragged_two_sizes_and_defocus(mods):
    eager, graphed = _pipes(mods)
    mols = _mols(mods, [12.0, 20.0, 16.0, 14.0])
    rois = [128, 128, 64, 128]
    dfs = [500.0, 600.0, 700.0, 800.0]
    ref = eager.run_batch(mols, defocus=dfs, rois=rois, to_host=True)
    for rep in range(5):
        assert _same(graphed.run_batch(mols, defocus=dfs, rois=rois, to_host=True), ref), rep
    # other defocus values are another structure (their phases are launch arguments)
    dfs2 = [900.0, 600.0, 700.0, 800.0]
    ref2 = eager.run_batch(mols, defocus=dfs2, rois=rois, to_host=True)
    for rep in range(5):
        assert _same(graphed.run_batch(mols, defocus=dfs2, rois=rois, to_host=True), ref2), rep
    assert not _same(ref, ref2)


def test_submit_batch_pipelined(mods):
    eager, graphed = _pipes(mods)
    batches = [_mols(mods, [16.0, 16.0]), _mols(mods, [14.0, 18.0])]
    refs = [eager.run_batch(b, to_host=True) for b in batches]
    pending = graphed.submit_batch(batches[0])
    for k in range(1, 8):
        nxt = graphed.submit_batch(batches[k % 2])
        assert _same(pending.result(), refs[(k - 1) % 2]), k
        pending = nxt
    assert _same(pending.result(), refs[1])


def test_chunked_route_replay(mods, monkeypatch):
    _, pipe, _ = mods
    monkeypatch.setattr(pipe, "_STACK_LIMIT_BYTES", 1 << 20)
    eager, graphed = _pipes(mods)
    mols = _mols(mods, [16.0, 16.0])
    ref = eager.run_batch(mols, to_host=True)
    for rep in range(5):
        assert _same(graphed.run_batch(mols, to_host=True), ref), rep
