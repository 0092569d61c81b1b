"""FP64 oracle of the off-grid ("smooth") projected potential and its coordinate
gradient (test infrastructure only).

emsim bins atoms to pixel centres before the Fourier-space build
(``SliceBuilder_kernel.cu:64-123``, ``SliceBuilder.cu:108-133``, band limit and clip of
``slice_builder_cuda.py:63-70, 88-99``), so its potential is piecewise constant in the
atom positions.  The smooth model keeps every step of that build but places each atom
at its exact lateral position: with the CUDA binning rule's start edge s0 and pixel d,
the continuous pixel coordinate is xi = (x - s0) / d - 1/2 (integer at a bin centre),
and the element's structure factor becomes

    S_e,s(k) = sum_a eps1_a(k1) eps2_a(k2),  eps(k) = exp(-2 pi i k xi / n)

with the Nyquist term (k = -n/2, n even) symmetrised to cos(pi xi), so that the
potential stays real.  V_s = clip(IFFT(sum_e T_e S_e,s), 1e-13) with T_e = F SF_e / N
the full-spectrum transfer of the reference build (scattering factor, band-limit round
trip, 1/N).  At bin centres the smooth potential equals the binned one; slice
membership (z) and the drop of atoms outside the box follow the binning rule, so the
z derivative is zero.
"""
from __future__ import annotations

import numpy as np
import scipy.fft as sfft

from .multislice import WORKERS, _cuda_axis_index, _element_of_rows, bandlimit_mask_half, cuda_bin_edges

__all__ = ["transfer_full", "atom_phases", "smooth_slices", "smooth_slices_grad"]


def transfer_full(sf_half: np.ndarray, n1: int, n2: int, bandlimit: bool = True) -> np.ndarray:
    """T_e(k) = F(k) SF_e(k) / N, (nE, n1, n2) float64.  F is the symmetric full-spectrum
    equivalent of irfft2(rfft2(V) * fil_half): (G(k) + G(-k)) / 2 with G the half mask
    weighted 1 on self-conjugate columns and 2 elsewhere."""
    h = n2 // 2 + 1
    if bandlimit:
        fil = bandlimit_mask_half(n1, n2).astype(np.float64)
        G = np.zeros((n1, n2))
        w = np.full(h, 2.0)
        w[0] = 1.0
        if n2 % 2 == 0:
            w[-1] = 1.0
        G[:, :h] = fil * w
        Gm = G[(-np.arange(n1)) % n1][:, (-np.arange(n2)) % n2]
        F = 0.5 * (G + Gm)
    else:
        F = np.ones((n1, n2))
    sf = np.asarray(sf_half, dtype=np.float64)
    ne = sf.shape[0]
    full = np.zeros((ne, n1, n2))
    full[:, :, :h] = sf
    j = np.arange(h, n2)
    full[:, :, h:] = sf[:, (-np.arange(n1)) % n1][:, :, n2 - j]
    return F[None] * full / float(n1 * n2)


def _freq(n: int) -> np.ndarray:
    return np.where(np.arange(n) < (n + 1) // 2, np.arange(n), np.arange(n) - n).astype(np.float64)


def atom_phases(coords, counts, n_slices, n1, n2, dz, d1, d2):
    """(element, slice, xi1, xi2, keep) of every row of coords (z, x, y) sorted by element;
    slice index and membership from the CUDA binning rule."""
    c = np.asarray(coords, dtype=np.float32).reshape(-1, 3)
    el = _element_of_rows(counts, c.shape[0])
    keep = el < len(counts)
    s, ins = _cuda_axis_index(c[:, 0], n_slices, dz)
    i1, in1 = _cuda_axis_index(c[:, 1], n1, d1)
    i2, in2 = _cuda_axis_index(c[:, 2], n2, d2)
    keep &= ins & in1 & in2
    _, s1, _ = cuda_bin_edges(n1, d1)
    _, s2, _ = cuda_bin_edges(n2, d2)
    xi1 = (c[:, 1].astype(np.float64) - float(s1)) / float(np.float32(d1)) - 0.5
    xi2 = (c[:, 2].astype(np.float64) - float(s2)) / float(np.float32(d2)) - 0.5
    return el, s, xi1, xi2, keep


def _eps(xi: np.ndarray, n: int):
    """eps (A, n) and d eps / d xi (A, n)."""
    k = _freq(n)
    e = np.exp(-2j * np.pi * np.outer(xi, k) / n)
    de = (-2j * np.pi * k / n)[None, :] * e
    if n % 2 == 0:
        ny = n // 2
        e[:, ny] = np.cos(np.pi * xi)
        de[:, ny] = -np.pi * np.sin(np.pi * xi)
    return e, de


def smooth_slices(coords, counts, n_slices, n1, n2, dz, d1, d2, T, xi_override=None):
    """V (n_slices, n1, n2) float64 of one molecule.  ``xi_override``: (xi1, xi2) in
    place of the float32-derived pixel coordinates (finite differences in FP64)."""
    el, s, xi1, xi2, keep = atom_phases(coords, counts, n_slices, n1, n2, dz, d1, d2)
    if xi_override is not None:
        xi1, xi2 = xi_override
    spec = np.zeros((n_slices, n1, n2), dtype=np.complex128)
    for e in range(len(counts)):
        for sl in range(n_slices):
            m = keep & (el == e) & (s == sl)
            if not m.any():
                continue
            e1, _ = _eps(xi1[m], n1)
            e2, _ = _eps(xi2[m], n2)
            spec[sl] += T[e] * (e1.T @ e2)
    w = sfft.ifft2(spec, norm="forward", workers=WORKERS).real
    return np.maximum(w, 1e-13)


def smooth_slices_grad(coords, counts, n_slices, n1, n2, dz, d1, d2, T, V, gV, xi_override=None):
    """dLoss/dcoords (n_atoms, 3) float64 for dLoss/dV = gV (columns z, x, y; z is 0)."""
    el, s, xi1, xi2, keep = atom_phases(coords, counts, n_slices, n1, n2, dz, d1, d2)
    if xi_override is not None:
        xi1, xi2 = xi_override
    gW = np.where(np.asarray(V) > 1e-13, gV, 0.0)
    # Gamma(k) = sum_p gW(p) exp(+2 pi i k.p / n) = conj(FFT(gW))(k) for real gW
    gam = np.conj(sfft.fft2(gW, workers=WORKERS))
    out = np.zeros((len(el), 3))
    for e in range(len(counts)):
        for sl in range(n_slices):
            m = keep & (el == e) & (s == sl)
            if not m.any():
                continue
            B = T[e] * gam[sl]
            e1, de1 = _eps(xi1[m], n1)
            e2, de2 = _eps(xi2[m], n2)
            M = B @ e2.T      # (n1, A)
            Md = B @ de2.T
            g1 = np.real(np.sum(de1.T * M, axis=0))
            g2 = np.real(np.sum(e1.T * Md, axis=0))
            out[m, 1] = g1 / float(np.float32(d1))
            out[m, 2] = g2 / float(np.float32(d2))
    return out
