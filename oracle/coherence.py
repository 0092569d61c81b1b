"""FP64 oracle of partially coherent imaging (test infrastructure only: imported by
tests/, never by the product path).

The reference has no partial coherence: its README lists the partially coherent CTF as
future work, so there is nothing of the reference to pin this restatement to.  It
restates the published treatment instead (J. Frank, "The envelope of electron
microscopic transfer functions for partially coherent illumination", Optik 38 (1973)
519-536; E. J. Kirkland, Advanced Computing in Electron Microscopy, chapter on the
transfer function and partial coherence):

* focal spread: the image is the incoherent average over a Gaussian distribution of
  defocus values (mean df, standard deviation sigma), evaluated with an n-point
  Gauss-Hermite rule: df_k = df + sqrt(2) sigma x_k, weights w_k / sqrt(pi);
* illumination semi-angle a: the quasi-coherent spatial envelope
  E_s(k) = exp(-(pi a / lambda)^2 (Cs lambda^3 k^3 - df lambda k)^2) multiplies the
  lens transfer exp(-i chi(k)) inside the aperture.

Parity is unpinned against the reference (it has no such feature).  The coherent lens
transfer is the oracle's FP64 "fftw" one (WavePropagator.cpp:105-138 restated in
oracle/multislice.py).
"""
from __future__ import annotations

import math

import numpy as np

from oracle import multislice as om


def quadrature(defocus: float, focal_spread: float, n: int = 7):
    """Gauss-Hermite defocus values and weights (sum 1) for a Gaussian focal spread."""
    if focal_spread == 0:
        return np.array([float(defocus)]), np.array([1.0])
    x, w = np.polynomial.hermite.hermgauss(int(n))
    return float(defocus) + math.sqrt(2.0) * float(focal_spread) * x, w / math.sqrt(math.pi)


def spatial_envelope(wp: om.WavePropagator, cs_mm: float, defocus: float, angle: float) -> np.ndarray:
    """E_s(k) on the unshifted FFT grid of ``wp`` (FP64)."""
    lam = float(wp.wave_length)
    f2 = np.asarray(wp.f2, dtype=np.float64)
    g = cs_mm * 1e7 * lam ** 3 * f2 - defocus * lam  # (Cs lambda^3 k^3 - df lambda k) / k
    return np.exp(-(math.pi * angle / lam) ** 2 * f2 * g * g)


def lens_intensity_incoherent(wp: om.WavePropagator, exit_wave, cs_mm: float, defocus_values, weights,
                              aperture: float, angle: float = 0.0) -> np.ndarray:
    """sum_k w_k |IFFT(FFT(psi) * exp(-i chi_k) * aperture * E_s,k)|^2 in FP64, for one
    (n1, n2) exit wave or a (B, n1, n2) stack."""
    psi = np.asarray(exit_wave, dtype=np.complex128)
    F = np.fft.fft2(psi, axes=(-2, -1))
    out = np.zeros(psi.shape, dtype=np.float64)
    for df, w in zip(np.atleast_1d(defocus_values), np.atleast_1d(weights)):
        hr, hi, keep = wp.lens_transfer(cs_mm, float(df), aperture)
        h = (hr + 1j * hi) * keep
        if angle > 0:
            h = h * spatial_envelope(wp, cs_mm, float(df), angle)
        g = np.fft.ifft2(F * h, axes=(-2, -1))
        out += w * (g.real ** 2 + g.imag ** 2)
    return out


def image_partially_coherent(n1: int, n2: int, d1: float, d2: float, kev: float, slices, dz: float, dose: float,
                             cs_mm: float, defocus: float, aperture: float, focal_spread: float, angle: float,
                             n_focal: int = 7) -> np.ndarray:
    """Plane wave -> FP64 multislice -> partially coherent lens intensity."""
    wp = om.WavePropagator(n1, n2, d1, d2, kev, "fftw", np.float64)
    psi = wp.multislice_propagate(wp.init_wave(dose).astype(np.complex128), np.asarray(slices, np.float64), dz)
    dfs, wts = quadrature(defocus, focal_spread, n_focal)
    return lens_intensity_incoherent(wp, psi, cs_mm, dfs, wts, aperture, angle)
