"""Seeded voxel water (test infrastructure only): a numpy model of the engine's
``emsim_gb300_add_water`` draws, against which the GPU counts are checked exactly.

The water rule is the reference's (``emsim/backend/slice_builder_base.py:134-147``): in
every voxel empty for all elements add Poisson(w) oxygens and Poisson(2 w) hydrogens,
w = water_num_dens * d1 * d2 * dz.  The random numbers follow Philox4x32-10 (Salmon,
Moraes, Dror, Shaw, SC11) with counter (voxel_lo, voxel_hi, stream, 0) and key
(seed_lo, seed_hi); word 0 -> oxygen, word 1 -> hydrogen; Poisson by sequential
inversion in float64.  ``tests/test_host_logic.py`` pins the Philox restatement to the
published known-answer vectors.
"""
from __future__ import annotations

import math

import numpy as np

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF
MAX_COUNT = 255


def philox4x32_10(counter, key):
    """Philox4x32-10 of one counter (4 uint32) and key (2 uint32) -> 4 uint32."""
    c = [int(x) & MASK for x in counter]
    k0, k1 = int(key[0]) & MASK, int(key[1]) & MASK
    for r in range(10):
        if r:
            k0 = (k0 + W0) & MASK
            k1 = (k1 + W1) & MASK
        p0 = M0 * c[0]
        p1 = M1 * c[2]
        c = [((p1 >> 32) ^ c[1] ^ k0) & MASK, p1 & MASK, ((p0 >> 32) ^ c[3] ^ k1) & MASK, p0 & MASK]
    return c


def philox_vec(v: np.ndarray, stream: int, seed: int):
    """Words 0 and 1 of Philox4x32-10 for counters (v_lo, v_hi, stream, 0), vectorised."""
    v = np.asarray(v, dtype=np.uint64)
    c0 = (v & np.uint64(MASK)).astype(np.uint64)
    c1 = (v >> np.uint64(32)).astype(np.uint64)
    c2 = np.full_like(c0, stream & MASK)
    c3 = np.zeros_like(c0)
    k0, k1 = np.uint64(seed & MASK), np.uint64((seed >> 32) & MASK)
    m = np.uint64(MASK)
    for r in range(10):
        if r:
            k0 = (k0 + np.uint64(W0)) & m
            k1 = (k1 + np.uint64(W1)) & m
        p0 = np.uint64(M0) * c0
        p1 = np.uint64(M1) * c2
        c0, c1, c2, c3 = ((p1 >> np.uint64(32)) ^ c1 ^ k0) & m, p1 & m, ((p0 >> np.uint64(32)) ^ c3 ^ k1) & m, p0 & m
    return c0.astype(np.uint32), c1.astype(np.uint32)


def poisson_inv(words: np.ndarray, lam: float) -> np.ndarray:
    """Smallest k with u < F_k, u = word * 2^-32, F the Poisson(lam) distribution
    function accumulated in float64 exactly as the device does."""
    u = words.astype(np.float64) * 2.3283064365386963e-10
    p = np.full(u.shape, math.exp(-lam))
    F = p.copy()
    k = np.zeros(u.shape, dtype=np.int64)
    active = u >= F
    for j in range(1, MAX_COUNT + 1):
        if not active.any():
            break
        p = np.where(active, p * lam / float(j), p)
        F = np.where(active, F + p, F)
        k = np.where(active, j, k)
        active = active & (u >= F)
    return k


def add_water(hist: np.ndarray, h_index: int, o_index: int, water_num_dens: float, d1: float, d2: float,
              dz: float, seed: int, stream: int = 0) -> np.ndarray:
    """hist (n_elems, n_slices, n1, n2) float32 -> hist with the seeded water added."""
    h = np.array(hist, dtype=np.float32, copy=True)
    ne = h.shape[0]
    flat = h.reshape(ne, -1)
    vac = np.all(flat == 0, axis=0)
    idx = np.nonzero(vac)[0]
    w = water_num_dens * d1 * d2 * dz
    wo, wh = philox_vec(idx, stream, seed)
    flat[o_index, idx] += poisson_inv(wo, w).astype(np.float32)
    flat[h_index, idx] += poisson_inv(wh, 2.0 * w).astype(np.float32)
    return h
