"""Seeded synthetic specimens for benchmarks and examples (emsim itself reads PDB files,
emsim/utils/pdb.py, which need a network; these stand in with the same atom mix).

* ``protein_blob``: C/N/O/S in fractions 0.63/0.17/0.19/0.01, uniform in a ball
  (radius * U^(1/3) along an isotropic direction), float32 (z, x, y).
* ``batching_mix``: the mixed batch of blobs with log-uniform atom counts, radius scaled
  to 0.1 atoms/A^3, a uniform random orientation (Shoemake quaternions, emsim/utils/rot.py
  :8-53) and, for every other blob, amorphous ice: O uniform at 0.0334 A^-3 over the
  field of view times the blob's z extent plus two H per O within 1 A.
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np

from .atoms import get_rotation_mattrices, random_uniform_quaternions

__all__ = ["protein_blob", "ice_layer", "batching_mix", "carbon_slab"]


def carbon_slab(seed: int = 0, lateral: float = 204.8, thickness: float = 200.0,
                density: float = 0.1) -> Tuple[np.ndarray, np.ndarray]:
    """Amorphous-carbon slab: round(density * lateral^2 * thickness) C atoms uniform over
    [-thickness/2, thickness/2) x [-lateral/2, lateral/2)^2, float32 (z, x, y).  The
    defaults give 838,861 atoms for a 2048^2 wave at 0.1 A with 400 slices of 0.5 A."""
    rng = np.random.default_rng(seed)
    n_atoms = int(round(density * lateral * lateral * thickness))
    lo = np.array([-thickness / 2, -lateral / 2, -lateral / 2])
    xyz = (lo + rng.random((n_atoms, 3)) * np.array([thickness, lateral, lateral])).astype(np.float32)
    return np.full(n_atoms, 6, dtype=np.int64), xyz


def protein_blob(n_atoms: int = 50_000, radius: float = 40.0, seed: int = 0) -> Tuple[np.ndarray, np.ndarray]:
    rng = np.random.default_rng(seed)
    el = rng.choice(np.array([6, 7, 8, 16]), size=n_atoms, p=[0.63, 0.17, 0.19, 0.01])
    v = rng.normal(size=(n_atoms, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    r = radius * rng.random(n_atoms) ** (1.0 / 3.0)
    return el, (v * r[:, None]).astype(np.float32)


def ice_layer(rng: np.random.Generator, lateral: float, z_lo: float, z_hi: float, o_density: float = 0.0334):
    """Amorphous ice in the box [z_lo, z_hi] x [-lateral/2, lateral/2)^2: Poisson number
    of O at o_density A^-3, uniform, and two H per O at uniform directions within 1 A."""
    vol = lateral * lateral * max(z_hi - z_lo, 0.0)
    n_o = int(rng.poisson(o_density * vol))
    lo = np.array([z_lo, -lateral / 2, -lateral / 2])
    hi = np.array([z_hi, lateral / 2, lateral / 2])
    o = lo + rng.random((n_o, 3)) * (hi - lo)
    d = rng.normal(size=(2 * n_o, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    h = np.repeat(o, 2, axis=0) + d * rng.random((2 * n_o, 1)) ** (1.0 / 3.0)
    el = np.concatenate([np.full(n_o, 8), np.full(2 * n_o, 1)])
    return el, np.concatenate([o, h]).astype(np.float32)


def batching_mix(n_blobs: int, seed: int = 0, pixel: float = 1.0, n_min: int = 5_000, n_max: int = 200_000,
                 density: float = 0.1) -> List[Tuple[np.ndarray, np.ndarray, int]]:
    """[(elements, coordinates, roi)] for n_blobs blobs; roi 256 or 512 with p = 1/2,
    every odd-numbered blob embedded in ice over its field of view."""
    rng = np.random.default_rng(seed)
    out = []
    quats = random_uniform_quaternions(n_blobs, rng)
    rots = get_rotation_mattrices(quats)
    for k in range(n_blobs):
        n = int(round(math.exp(rng.uniform(math.log(n_min), math.log(n_max)))))
        radius = (3.0 * n / (4.0 * math.pi * density)) ** (1.0 / 3.0)
        el, xyz = protein_blob(n, radius, int(rng.integers(1 << 31)))
        xyz = (xyz.astype(np.float64) @ rots[k].T).astype(np.float32)
        roi = 256 if rng.random() < 0.5 else 512
        if k % 2 == 1:
            e2, x2 = ice_layer(rng, roi * pixel, float(xyz[:, 0].min()), float(xyz[:, 0].max()))
            el = np.concatenate([el, e2])
            xyz = np.concatenate([xyz, x2])
        out.append((el, xyz, roi))
    return out
