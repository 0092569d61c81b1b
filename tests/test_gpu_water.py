"""Seeded voxel water on the GPU (emsim_gb300_add_water) against the numpy model of the
same Philox draws (exact), plus the statistics of the reference's rule (mean counts)."""
import numpy as np
import pytest

from oracle import water as ow

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import backend, physics
    return backend, physics


def test_water_matches_model_exactly(eng):
    backend, physics = eng
    zs, ns, n, dz, d = [1, 6, 8], 6, 64, 2.0, 1.0
    rng = np.random.default_rng(2)
    hist = np.zeros((3, ns, n, n), np.float32)
    occ = rng.random((ns, n, n)) < 0.2
    hist[1][occ] = rng.integers(1, 4, size=occ.sum())
    b = backend.MultiSlicesBuilder(zs, ns, n, n, dz, d, d)
    got = np.asarray(b.add_water(hist.copy(), seed=1234567, stream_id=5).get())
    ref = ow.add_water(hist, 0, 2, physics.water_num_dens, d, d, dz, seed=1234567, stream=5)
    np.testing.assert_array_equal(got, ref)
    # occupied voxels untouched, only H and O change
    np.testing.assert_array_equal(got[:, occ], hist[:, occ])
    np.testing.assert_array_equal(got[1], hist[1])
    # deterministic; another seed differs
    again = np.asarray(b.add_water(hist.copy(), seed=1234567, stream_id=5).get())
    np.testing.assert_array_equal(again, got)
    other = np.asarray(b.add_water(hist.copy(), seed=7, stream_id=5).get())
    assert not np.array_equal(other, got)


def test_water_statistics(eng):
    backend, physics = eng
    zs, ns, n, dz, d = [1, 8], 40, 256, 2.0, 1.0
    b = backend.MultiSlicesBuilder(zs, ns, n, n, dz, d, d)
    got = np.asarray(b.add_water(np.zeros((2, ns, n, n), np.float32), seed=42).get())
    w = physics.water_num_dens * d * d * dz
    nv = ns * n * n
    for idx, lam in ((1, w), (0, 2 * w)):
        m = got[idx].mean()
        assert abs(m - lam) < 5 * np.sqrt(lam / nv), (idx, m, lam)
        assert abs(got[idx].var() - lam) < 0.02 * lam
