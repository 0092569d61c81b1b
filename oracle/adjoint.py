"""FP64 oracle of the differentiable image and its adjoint (test infrastructure only).

emsim forms images without derivatives; the forward restated here is the reference's
native image chain (multislice ``WavePropagator.cu:62-70`` with the 2/3 band limit of
``WavePropagator_kernel.cu:46-94``, lens ``WavePropagator_kernel.cu:97-145``, intensity
``pipe.py:81-82``), evaluated in complex128 through ``oracle.multislice`` 's transfer
functions.  The adjoint is the textbook reverse sweep of that chain:

    lambda_u = g u,   lambda_S = L^H lambda_u,
    mu_s = P^H lambda_{s+1},   dLoss/dV_s = 2 sigma Im(mu_s conj(phi_s)),
    lambda_s = conj(t_s) mu_s,

with phi_s = psi_s t_s the transmitted wave and g = dLoss/dI.  Nothing here is
checkpointed: every phi_s is kept.  ``tests/test_adjoint_oracle.py`` pins this adjoint
against torch complex128 autograd of the same forward and against FP64 central
differences.
"""
from __future__ import annotations

import numpy as np
import scipy.fft as sfft

from .multislice import WORKERS, WavePropagator

__all__ = ["ImageChain", "loss_weighted"]


class ImageChain:
    """FP64 forward/adjoint of I = |L P t_{S-1} ... P t_0 psi_0|^2 for one geometry."""

    def __init__(self, n1: int, n2: int, d1: float, d2: float, beam_energy_kev: float):
        self.wp = WavePropagator(n1, n2, d1, d2, beam_energy_kev, semantics="fftw", dtype=np.float64)
        self.n1, self.n2 = n1, n2
        self.sigma = float(self.wp.wave_length * self.wp.relativity_gamma)

    def _prop(self, dz: float) -> np.ndarray:
        pr, pi, keep = self.wp._propagator(dz)
        return np.where(keep, pr + 1j * pi, 0)

    def _lens(self, cs_mm: float, defocus: float, aperture: float) -> np.ndarray:
        hr, hi, keep = self.wp.lens_transfer(cs_mm, defocus, aperture)
        return np.where(keep, hr + 1j * hi, 0)

    @staticmethod
    def _f(x):
        return sfft.fft2(x, workers=WORKERS)

    @staticmethod
    def _fi(x):
        return sfft.ifft2(x, workers=WORKERS)

    def _stack(self, slices, b):
        s = np.asarray(slices, dtype=np.float64)
        return s[b] if s.ndim == 4 else s

    def forward(self, slices, dz, dose, cs_mm, defocus, aperture, nb, keep_phi=False):
        """images (nb, n1, n2); with keep_phi also (u, phi) for the adjoint."""
        dfs = np.atleast_1d(np.asarray(defocus, dtype=np.float64))
        H = self._prop(dz)
        amp = complex(self.wp.init_wave(dose)[0, 0])  # complex64 plane wave (wave_propagator_base.py:25-29)
        imgs, us, phis = [], [], []
        for b in range(nb):
            v = self._stack(slices, b)
            psi = np.full((self.n1, self.n2), amp, dtype=np.complex128)
            ph = []
            for s in range(v.shape[0]):
                phi = psi * np.exp(1j * self.sigma * v[s])
                if keep_phi:
                    ph.append(phi)
                psi = self._fi(self._f(phi) * H)
            u = self._fi(self._f(psi) * self._lens(cs_mm, dfs[b % len(dfs)], aperture))
            imgs.append(u.real ** 2 + u.imag ** 2)
            us.append(u)
            phis.append(ph)
        imgs = np.stack(imgs)
        return (imgs, us, phis) if keep_phi else imgs

    def adjoint(self, slices, dz, dose, cs_mm, defocus, aperture, nb, grad_image):
        """dLoss/dV for dLoss/dI = grad_image: shape of ``slices`` (shared stacks get
        the sum over the nb images)."""
        dfs = np.atleast_1d(np.asarray(defocus, dtype=np.float64))
        s_all = np.asarray(slices, dtype=np.float64)
        _, us, phis = self.forward(slices, dz, dose, cs_mm, defocus, aperture, nb, keep_phi=True)
        Hc = np.conj(self._prop(dz))
        grad = np.zeros_like(s_all)
        g = np.asarray(grad_image, dtype=np.float64).reshape(nb, self.n1, self.n2)
        for b in range(nb):
            v = self._stack(s_all, b)
            lam = self._fi(self._f(g[b] * us[b]) * np.conj(self._lens(cs_mm, dfs[b % len(dfs)], aperture)))
            gb = grad[b] if s_all.ndim == 4 else grad
            for s in range(v.shape[0] - 1, -1, -1):
                mu = self._fi(self._f(lam) * Hc)
                gb[s] += 2.0 * self.sigma * np.imag(mu * np.conj(phis[b][s]))
                lam = np.conj(np.exp(1j * self.sigma * v[s])) * mu
        return grad


def loss_weighted(images: np.ndarray, weights: np.ndarray) -> float:
    """Loss = sum(weights * images): its dLoss/dI is ``weights``."""
    return float(np.sum(np.asarray(weights, dtype=np.float64) * images))
