"""GPU off-grid ("smooth") slices and their coordinate adjoint against the FP64 smooth
oracle (oracle/smooth.py), and the full chain coordinates -> slices -> image -> loss
against FP64 central differences.

Tolerances: smooth slices relative L2 <= 1e-5 against the FP64 oracle (and <= 1e-5
against the binned build for atoms at bin centres); coordinate gradient for a given
dLoss/dV relative L2 <= GRAD_TOL against the FP64 analytic gradient; full chain
directional derivative within CHAIN_TOL of FP64 central differences (h = 1e-4 A),
limited by the float32 image: the loss depends on I - I_target, a 1e-3 fraction of I.
"""
import numpy as np
import pytest

from oracle import multislice as om
from oracle import smooth as osm
from oracle.adjoint import ImageChain

pytestmark = pytest.mark.gpu

GRAD_TOL = 1e-5
CHAIN_TOL = 5e-3


@pytest.fixture(scope="module")
def eng():
    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import autograd, backend
    return backend, autograd


def _mol(seed, n_atoms, zs, ns, n, dz, d, centred=False):
    rng = np.random.default_rng(seed)
    el = rng.choice(np.array(zs), size=n_atoms)
    if centred:
        _, s0, _ = om.cuda_bin_edges(n, d)
        ij = rng.integers(1, n - 1, size=(n_atoms, 2))
        z = (rng.random(n_atoms) * 2 - 1) * ns * dz / 2 * 0.95
        xyz = np.column_stack([z, float(s0) + (ij + 0.5) * d]).astype(np.float32)
    else:
        half = np.array([ns * dz / 2 * 0.95, n * d / 2 * 0.9, n * d / 2 * 0.9])
        xyz = ((rng.random((n_atoms, 3)) * 2 - 1) * half).astype(np.float32)
    _, xyz_s, _, cnt = om.sort_elements_and_count(el, xyz, zs)
    return xyz_s, cnt


CASES = [(64, 6, 1.0, 0.5, 300, (6, 8)), (128, 9, 2.0, 0.5, 2000, (6, 7, 8, 16)), (256, 4, 2.0, 1.0, 5000, (6, 8, 16)),
         (32, 3, 1.0, 0.25, 50, (29,))]


@pytest.mark.parametrize("n,ns,dz,d,n_atoms,zs", CASES)
def test_smooth_slices_match_fp64_oracle(eng, n, ns, dz, d, n_atoms, zs):
    import torch
    backend, autograd = eng
    zs = list(zs)
    xyz, cnt = _mol(n + ns, n_atoms, zs, ns, n, dz, d)
    b = backend.MultiSlicesBuilder(zs, ns, n, n, dz, d, d)
    got = autograd.smooth_slices(b, torch.tensor(xyz, device="cuda"), cnt).cpu().numpy()
    T = osm.transfer_full(om.scattering_factors_half(zs, n, n, d, d), n, n)
    ref = osm.smooth_slices(xyz, cnt, ns, n, n, dz, d, d, T)
    assert got.shape == (ns, n, n)
    assert om.rel_l2(got, ref) < 1e-5
    # deterministic
    again = autograd.smooth_slices(b, torch.tensor(xyz, device="cuda"), cnt).cpu().numpy()
    np.testing.assert_array_equal(again, got)


def test_smooth_equals_binned_at_bin_centres(eng):
    import torch
    backend, autograd = eng
    zs, ns, n, dz, d = [6, 7, 8, 16], 8, 128, 2.0, 0.5
    xyz, cnt = _mol(3, 1500, zs, ns, n, dz, d, centred=True)
    b = backend.MultiSlicesBuilder(zs, ns, n, n, dz, d, d)
    got = autograd.smooth_slices(b, torch.tensor(xyz, device="cuda"), cnt).cpu().numpy()
    binned = np.asarray(backend.build_slices_batch(b, [(xyz, cnt)]).get())[0]
    assert om.rel_l2(got, binned) < 1e-5


def test_smooth_batch_equals_single(eng):
    import torch
    backend, autograd = eng
    zs, ns, n, dz, d = [6, 8], 5, 64, 1.0, 0.5
    mols = [_mol(10 + k, 200 + 100 * k, zs, ns, n, dz, d) for k in range(3)]
    b = backend.MultiSlicesBuilder(zs, ns, n, n, dz, d, d)
    xyz = torch.tensor(np.concatenate([m[0] for m in mols]), device="cuda")
    got = autograd.smooth_slices(b, xyz, np.stack([m[1] for m in mols])).cpu().numpy()
    for k, (c, cnt) in enumerate(mols):
        one = autograd.smooth_slices(b, torch.tensor(c, device="cuda"), cnt).cpu().numpy()
        np.testing.assert_array_equal(got[k], one)


@pytest.mark.parametrize("n,ns,dz,d,n_atoms,zs", CASES[:3])
def test_smooth_coordinate_gradient_matches_fp64(eng, n, ns, dz, d, n_atoms, zs):
    import torch
    backend, autograd = eng
    zs = list(zs)
    xyz, cnt = _mol(7 * n + ns, n_atoms, zs, ns, n, dz, d)
    b = backend.MultiSlicesBuilder(zs, ns, n, n, dz, d, d)
    c = torch.tensor(xyz, device="cuda", requires_grad=True)
    v = autograd.smooth_slices(b, c, cnt)
    w = np.random.default_rng(1).standard_normal((ns, n, n)).astype(np.float32)
    (v * torch.tensor(w, device="cuda")).sum().backward()
    got = c.grad.cpu().numpy()
    T = osm.transfer_full(om.scattering_factors_half(zs, n, n, d, d), n, n)
    # the clip's derivative is taken where the float32 slices are above 1e-13; pixels whose
    # exact potential lies within float32 rounding of zero are ambiguous, so the FP64
    # gradient uses the same mask
    vg = v.detach().cpu().numpy().astype(np.float64)
    ref = osm.smooth_slices_grad(xyz, cnt, ns, n, n, dz, d, d, T, vg, w.astype(np.float64))
    assert np.all(got[:, 0] == 0)
    err = om.rel_l2(got, ref)
    assert err < GRAD_TOL, err


def test_full_chain_coordinate_gradient_central_differences(eng):
    """coords -> smooth slices -> multislice image (several defocus values) -> MSE to the
    image of a jittered copy; FP64 central differences with h = 1e-4 A."""
    import torch
    backend, autograd = eng
    zs, ns, n, dz, d, kev = [6, 7, 8, 16], 8, 128, 2.0, 0.5, 300.0
    el, xyz0 = om.protein_blob(1500, radius=7.0, seed=4)
    rng = np.random.default_rng(5)
    _, xyz, _, cnt = om.sort_elements_and_count(el, xyz0, zs)
    jit = (xyz + rng.normal(scale=0.2, size=xyz.shape)).astype(np.float32)
    dfs = [500.0, 1100.0]
    b = backend.MultiSlicesBuilder(zs, ns, n, n, dz, d, d)
    wp = backend.WavePropagator(n, n, d, d, kev)
    with torch.no_grad():
        target = autograd.image(wp, autograd.smooth_slices(b, torch.tensor(jit, device="cuda"), cnt), dz, 20.0, 1.0,
                                dfs, 12e-3)
    c = torch.tensor(xyz, device="cuda", requires_grad=True)
    img = autograd.image(wp, autograd.smooth_slices(b, c, cnt), dz, 20.0, 1.0, dfs, 12e-3)
    loss = torch.mean((img - target) ** 2)
    loss.backward()
    g = c.grad.cpu().numpy().astype(np.float64)
    T = osm.transfer_full(om.scattering_factors_half(zs, n, n, d, d), n, n)
    chain = ImageChain(n, n, d, d, kev)
    tgt = target.cpu().numpy().astype(np.float64)
    _, _, xi1, xi2, _ = osm.atom_phases(xyz, cnt, ns, n, n, dz, d, d)

    def loss64(dx):
        v = osm.smooth_slices(xyz, cnt, ns, n, n, dz, d, d, T, xi_override=(xi1 + dx[:, 0] / d, xi2 + dx[:, 1] / d))
        im = chain.forward(v, dz, 20.0, 1.0, dfs, 12e-3, len(dfs))
        return float(np.mean((im - tgt) ** 2))

    h = 1e-4
    dirn = np.random.default_rng(6).standard_normal((len(xyz), 2))
    fd = (loss64(h * dirn) - loss64(-h * dirn)) / (2 * h)
    an = float(np.sum(g[:, 1] * dirn[:, 0] + g[:, 2] * dirn[:, 1]))
    assert abs(fd - an) <= CHAIN_TOL * abs(fd), (fd, an)
