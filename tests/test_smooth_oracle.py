"""The smooth (off-grid) potential oracle (oracle/smooth.py): its transfer function
reproduces the binned build, it equals the binned potential for atoms at bin centres,
and its analytic coordinate gradient matches FP64 central differences (CPU)."""
import numpy as np

from oracle import multislice as om
from oracle import smooth as osm

ZS = [6, 8]
NS, N, DZ, D = 4, 32, 2.0, 0.5


def _atoms(seed, n_atoms=40, centred=False):
    rng = np.random.default_rng(seed)
    el = rng.choice(np.array(ZS), size=n_atoms)
    if centred:
        _, s0, _ = om.cuda_bin_edges(N, D)
        i = rng.integers(2, N - 2, size=(n_atoms, 2))
        xy = float(s0) + (i + 0.5) * D
        z = (rng.random(n_atoms) * 2 - 1) * NS * DZ / 2 * 0.9
        xyz = np.column_stack([z, xy]).astype(np.float32)
    else:
        half = np.array([NS * DZ / 2 * 0.9, N * D / 2 * 0.8, N * D / 2 * 0.8])
        xyz = ((rng.random((n_atoms, 3)) * 2 - 1) * half).astype(np.float32)
    _, xyz_s, uz, cnt = om.sort_elements_and_count(el, xyz, ZS)
    return xyz_s, cnt


def _T():
    sf = om.scattering_factors_half(ZS, N, N, D, D)
    return sf, osm.transfer_full(sf, N, N)


def test_transfer_reproduces_binned_build():
    xyz, cnt = _atoms(1)
    sf, T = _T()
    hist = om.bin_atoms_cuda(xyz, cnt, (NS, N, N), (DZ, D, D)).astype(np.float64)
    ref = om.make_slices(hist, sf, "fftw", np.float64)
    spec = np.einsum("ekl,eskl->skl", T, np.fft.fft2(hist))
    got = np.maximum(np.fft.ifft2(spec, norm="forward").real, 1e-13)
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


def test_smooth_equals_binned_at_bin_centres():
    xyz, cnt = _atoms(2, centred=True)
    sf, T = _T()
    hist = om.bin_atoms_cuda(xyz, cnt, (NS, N, N), (DZ, D, D)).astype(np.float64)
    ref = om.make_slices(hist, sf, "fftw", np.float64)
    got = osm.smooth_slices(xyz, cnt, NS, N, N, DZ, D, D, T)
    np.testing.assert_allclose(got, ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


def test_smooth_is_real_and_periodic_nyquist_consistent():
    xyz, cnt = _atoms(3)
    _, T = _T()
    el, s, xi1, xi2, keep = osm.atom_phases(xyz, cnt, NS, N, N, DZ, D, D)
    v = osm.smooth_slices(xyz, cnt, NS, N, N, DZ, D, D, T)
    # shifting every atom by one whole pixel rolls the potential by one pixel
    v1 = osm.smooth_slices(xyz, cnt, NS, N, N, DZ, D, D, T, xi_override=(xi1 + 1.0, xi2))
    np.testing.assert_allclose(v1, np.roll(v, 1, axis=1), rtol=1e-9, atol=1e-12 * np.abs(v).max())


def test_smooth_gradient_matches_central_differences():
    xyz, cnt = _atoms(4)
    _, T = _T()
    el, s, xi1, xi2, keep = osm.atom_phases(xyz, cnt, NS, N, N, DZ, D, D)
    rng = np.random.default_rng(5)
    w = rng.standard_normal((NS, N, N))
    v = osm.smooth_slices(xyz, cnt, NS, N, N, DZ, D, D, T)
    g = osm.smooth_slices_grad(xyz, cnt, NS, N, N, DZ, D, D, T, v, w)
    assert np.all(g[:, 0] == 0)
    assert np.all(g[~keep] == 0)
    h = 1e-4  # Angstrom
    for _ in range(2):
        dx = rng.standard_normal((len(xi1), 2))
        lp = np.sum(w * osm.smooth_slices(xyz, cnt, NS, N, N, DZ, D, D, T,
                                          xi_override=(xi1 + h * dx[:, 0] / D, xi2 + h * dx[:, 1] / D)))
        lm = np.sum(w * osm.smooth_slices(xyz, cnt, NS, N, N, DZ, D, D, T,
                                          xi_override=(xi1 - h * dx[:, 0] / D, xi2 - h * dx[:, 1] / D)))
        fd = (lp - lm) / (2 * h)
        an = float(np.sum(g[:, 1] * dx[:, 0] + g[:, 2] * dx[:, 1]))
        assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)
