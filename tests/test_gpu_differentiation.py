"""The differentiation workload: 20,000 C/N/O/S atoms in a 50 A ball (atoms beyond the
64 slices of 1 A are dropped by the binning rule), 512 x 512 at 0.5 A, defocus uniform
in 300-1500 A, loss = MSE against the image of a copy jittered by 0.2 A.  Gradients with
respect to the slice potentials and the atom coordinates (off-grid slices) run on the
GPU with sqrt(N) checkpointing; 4 defocus values are checked against the FP64 adjoint
and FP64 central differences (h = 1e-4 A), the full batch of 32 for determinism.

Tolerances: dLoss/dV relative L2 <= 5e-5 against the FP64 adjoint given the same
dLoss/dI; coordinate directional derivative within 5e-3 of FP64 central differences
(the float32 image carries ~1e-6 relative error while I - I_target is ~1e-3 of I).
"""
import numpy as np
import pytest

from oracle import multislice as om
from oracle import smooth as osm
from oracle.adjoint import ImageChain

pytestmark = pytest.mark.gpu

N, NS, D, DZ, KEV, CS, AP, DOSE = 512, 64, 0.5, 1.0, 200.0, 1.3, 10e-3, 20.0
ZS = [6, 7, 8, 16]


@pytest.fixture(scope="module")
def setup():
    import torch

    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import autograd, backend
    el, xyz0 = om.protein_blob(20_000, radius=50.0, seed=77)
    rng = np.random.default_rng(78)
    _, xyz, _, cnt = om.sort_elements_and_count(el, xyz0, ZS)
    jit = (xyz + rng.normal(scale=0.2, size=xyz.shape)).astype(np.float32)
    dfs = rng.uniform(300.0, 1500.0, size=32)
    bld = backend.MultiSlicesBuilder(ZS, NS, N, N, DZ, D, D)
    wp = backend.WavePropagator(N, N, D, D, KEV)
    return torch, autograd, bld, wp, xyz, jit, cnt, dfs


def _forward_backward(torch, autograd, bld, wp, xyz, jit, cnt, dfs):
    with torch.no_grad():
        target = autograd.image(wp, autograd.smooth_slices(bld, torch.tensor(jit, device="cuda"), cnt), DZ, DOSE, CS,
                                list(dfs), AP)
    c = torch.tensor(xyz, device="cuda", requires_grad=True)
    v = autograd.smooth_slices(bld, c, cnt)
    v.retain_grad()
    img = autograd.image(wp, v, DZ, DOSE, CS, list(dfs), AP)
    loss = torch.mean((img - target) ** 2)
    loss.backward()
    return target, c, v, img, loss


def test_full_batch_runs_and_is_deterministic(setup):
    torch, autograd, bld, wp, xyz, jit, cnt, dfs = setup
    _, c1, v1, img1, l1 = _forward_backward(torch, autograd, bld, wp, xyz, jit, cnt, dfs)
    _, c2, v2, img2, l2 = _forward_backward(torch, autograd, bld, wp, xyz, jit, cnt, dfs)
    assert img1.shape == (32, N, N)
    assert torch.isfinite(c1.grad).all() and torch.isfinite(v1.grad).all()
    assert float(l1.detach()) == float(l2.detach())
    assert torch.equal(c1.grad, c2.grad) and torch.equal(v1.grad, v2.grad)
    kept = osm.atom_phases(xyz, cnt, NS, N, N, DZ, D, D)[4]
    g = c1.grad.cpu().numpy()
    assert np.all(g[~kept] == 0) and np.all(g[:, 0] == 0)
    assert np.count_nonzero(g[kept]) > 0.9 * 2 * kept.sum()


def test_gradients_against_fp64(setup):
    torch, autograd, bld, wp, xyz, jit, cnt, dfs_all = setup
    dfs = dfs_all[:4]
    target, c, v, img, _ = _forward_backward(torch, autograd, bld, wp, xyz, jit, cnt, dfs)
    chain = ImageChain(N, N, D, D, KEV)
    # slice potentials: FP64 adjoint for the same dLoss/dI
    g = (2.0 * (img.detach() - target) / img.numel()).cpu().numpy().astype(np.float64)
    v64 = v.detach().cpu().numpy().astype(np.float64)
    g64 = chain.adjoint(v64, DZ, DOSE, CS, dfs, AP, len(dfs), g)
    assert om.rel_l2(v.grad.cpu().numpy(), g64) < 5e-5
    # coordinates: FP64 central differences of the whole chain
    T = osm.transfer_full(om.scattering_factors_half(ZS, N, N, D, D), N, N)
    tgt = target.cpu().numpy().astype(np.float64)
    _, _, xi1, xi2, kept = osm.atom_phases(xyz, cnt, NS, N, N, DZ, D, D)

    def loss64(dx):
        vv = osm.smooth_slices(xyz, cnt, NS, N, N, DZ, D, D, T, xi_override=(xi1 + dx[:, 0] / D, xi2 + dx[:, 1] / D))
        im = chain.forward(vv, DZ, DOSE, CS, dfs, AP, len(dfs))
        return float(np.mean((im - tgt) ** 2))

    h = 1e-4
    dirn = np.random.default_rng(80).standard_normal((len(xyz), 2))
    fd = (loss64(h * dirn) - loss64(-h * dirn)) / (2 * h)
    gc = c.grad.cpu().numpy().astype(np.float64)
    an = float(np.sum(gc[:, 1] * dirn[:, 0] + gc[:, 2] * dirn[:, 1]))
    assert abs(fd - an) <= 5e-3 * abs(fd), (fd, an)
