"""Kirkland electron scattering factors (emsim/elem.py:120-156, 267-354).

f_e(q) = sum_i a_i / (q^2 + b_i) + c_i exp(-d_i q^2), zero for q^2 >= 16, on the
fftshifted fftfreq grid, with the parameters rounded to float32 as the reference does.
Results are cached per (elements, grid) because builders are created per image.
"""
from __future__ import annotations

import functools
from pathlib import Path
from typing import Sequence, Tuple

import numpy as np

_TABLE = Path(__file__).resolve().parent / "data" / "kirkland_fe_params.csv"


@functools.lru_cache(maxsize=1)
def _params_table() -> np.ndarray:
    return np.loadtxt(_TABLE, delimiter=",", comments="#", dtype=np.float64)


def elem_params(elem_numbers: Sequence[int]) -> np.ndarray:
    """(n, 12) float32 rows a1..a3, b1..b3, c1..c3, d1..d3 (elem.py:294-309)."""
    if not all(1 <= int(z) <= 103 for z in elem_numbers):
        raise ValueError("z must be a interger in range [1, 92]")
    tab = _params_table()
    return np.array([tab[int(z) - 1, 1:] for z in elem_numbers], dtype=np.float32)


def scattering_factors2d(elem_numbers: Sequence[int], n1: int, n2: int, d1: float, d2: float) -> np.ndarray:
    """(nE, n1, n2) float32 on the fftshifted grid (elem.py:267-291)."""
    kx = np.fft.fftshift(np.fft.fftfreq(n1, d1))
    ky = np.fft.fftshift(np.fft.fftfreq(n2, d2))
    kx, ky = np.meshgrid(kx, ky, indexing="ij")
    k = np.sqrt(kx * kx + ky * ky)
    q2 = k * k
    mask = q2 < 16
    pms = elem_params(elem_numbers)
    out = np.empty((len(elem_numbers), n1, n2), dtype=np.float32)
    for e in range(len(elem_numbers)):
        a, b, c, d = pms[e, 0:3], pms[e, 3:6], pms[e, 6:9], pms[e, 9:12]
        v = np.sum([a[i] / (q2 + b[i]) + c[i] * np.exp(-d[i] * q2) for i in range(3)], axis=0)
        out[e] = np.where(mask, v, 0.)
    return out


@functools.lru_cache(maxsize=64)
def _half_cached(key: Tuple[int, ...], n1: int, n2: int, d1: float, d2: float) -> np.ndarray:
    sf = scattering_factors2d(list(key), n1, n2, d1, d2)
    sf = np.fft.ifftshift(sf, axes=(-2, -1))
    out = np.ascontiguousarray(sf[:, :, :n2 // 2 + 1], dtype=np.float32)
    out.setflags(write=False)
    return out


def scattering_factors_half(unique_elements: Sequence[int], n1: int, n2: int, d1: float, d2: float) -> np.ndarray:
    """Builder layout (slice_builder_base.py:28-33): sorted elements, ifftshifted,
    first n2//2+1 columns, float32 (nE, n1, n2//2+1).  Read-only cached array."""
    return _half_cached(tuple(sorted(int(z) for z in unique_elements)), int(n1), int(n2), float(d1), float(d2))
