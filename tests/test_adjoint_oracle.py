"""The FP64 adjoint oracle (oracle/adjoint.py) against torch complex128 autograd of the
same forward and against FP64 central differences (CPU)."""
import numpy as np
import pytest
import torch

from oracle.adjoint import ImageChain, loss_weighted

N1, N2, D, KEV = 32, 32, 1.0, 200.0
DZ, DOSE, CS, AP = 2.0, 20.0, 1.3, 10e-3


def _case(seed=0, ns=5, nb=2, per_image=False):
    rng = np.random.default_rng(seed)
    shape = (nb, ns, N1, N2) if per_image else (ns, N1, N2)
    v = rng.uniform(0.0, 200.0, size=shape)
    w = rng.standard_normal((nb, N1, N2))
    dfs = rng.uniform(300.0, 1500.0, size=nb)
    return v, w, dfs


def _torch_grad(chain, v, w, dfs, nb):
    vt = torch.tensor(v, dtype=torch.float64, requires_grad=True)
    H = torch.tensor(chain._prop(DZ))
    amp = complex(chain.wp.init_wave(DOSE)[0, 0])
    loss = 0
    for b in range(nb):
        vb = vt[b] if vt.dim() == 4 else vt
        psi = torch.full((N1, N2), amp, dtype=torch.complex128)
        for s in range(vb.shape[0]):
            psi = torch.fft.ifft2(torch.fft.fft2(psi * torch.exp(1j * chain.sigma * vb[s])) * H)
        L = torch.tensor(chain._lens(CS, dfs[b], AP))
        u = torch.fft.ifft2(torch.fft.fft2(psi) * L)
        loss = loss + (torch.tensor(w[b]) * (u.real ** 2 + u.imag ** 2)).sum()
    loss.backward()
    return vt.grad.numpy(), float(loss.detach())


@pytest.mark.parametrize("per_image", [False, True])
def test_adjoint_matches_torch_autograd(per_image):
    nb = 2
    v, w, dfs = _case(per_image=per_image, nb=nb)
    chain = ImageChain(N1, N2, D, D, KEV)
    g = chain.adjoint(v, DZ, DOSE, CS, dfs, AP, nb, w)
    gt, loss_t = _torch_grad(chain, v, w, dfs, nb)
    loss = loss_weighted(chain.forward(v, DZ, DOSE, CS, dfs, AP, nb), w)
    assert abs(loss - loss_t) <= 1e-12 * abs(loss_t)
    assert g.shape == v.shape
    err = np.linalg.norm(g - gt) / np.linalg.norm(gt)
    assert err < 1e-11, err


def test_adjoint_matches_central_differences():
    nb = 2
    v, w, dfs = _case(seed=3, nb=nb)
    chain = ImageChain(N1, N2, D, D, KEV)
    g = chain.adjoint(v, DZ, DOSE, CS, dfs, AP, nb, w)
    rng = np.random.default_rng(7)
    for _ in range(3):
        d = rng.standard_normal(v.shape)
        h = 1e-3
        lp = loss_weighted(chain.forward(v + h * d, DZ, DOSE, CS, dfs, AP, nb), w)
        lm = loss_weighted(chain.forward(v - h * d, DZ, DOSE, CS, dfs, AP, nb), w)
        fd = (lp - lm) / (2 * h)
        an = float(np.sum(g * d))
        assert abs(fd - an) <= 1e-6 * abs(an), (fd, an)
    # single pixels of the first and last slice
    for (s, i, j) in [(0, 3, 5), (v.shape[0] - 1, 17, 30)]:
        d = np.zeros_like(v)
        d[s, i, j] = 1.0
        h = 1e-2
        lp = loss_weighted(chain.forward(v + h * d, DZ, DOSE, CS, dfs, AP, nb), w)
        lm = loss_weighted(chain.forward(v - h * d, DZ, DOSE, CS, dfs, AP, nb), w)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[s, i, j]) <= 1e-6 * max(abs(g[s, i, j]), 1e-3 * np.abs(g).max()), (fd, g[s, i, j])


def test_shared_stack_gradient_is_sum_over_images():
    nb = 3
    v, w, dfs = _case(seed=5, nb=nb)
    chain = ImageChain(N1, N2, D, D, KEV)
    g_shared = chain.adjoint(v, DZ, DOSE, CS, dfs, AP, nb, w)
    v4 = np.broadcast_to(v, (nb,) + v.shape).copy()
    g4 = chain.adjoint(v4, DZ, DOSE, CS, dfs, AP, nb, w)
    np.testing.assert_allclose(g_shared, g4.sum(axis=0), rtol=1e-12, atol=1e-12 * np.abs(g4).max())
