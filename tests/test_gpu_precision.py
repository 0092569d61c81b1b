"""Precision workload: amorphous-carbon slab, C atoms uniform at 0.1 A^-3 over
204.8 x 204.8 x 200 A (838,861 atoms), 2048 x 2048 wave at pixel 0.1 A, 400 slices of
0.5 A, 300 keV, Cs 1.0 mm, Scherzer defocus and aperture.  The GPU's plain FP32 path
(histogram-free slice build, fused multislice, lens, |psi|^2) is compared with the FP64
oracle run slab by slab (16 slices at a time, so the oracle holds ~0.5 GB).

Tolerance: relative L2 <= 1e-5 on the image and on the exit wave; the error is printed
(run with -s) together with the error on I - mean(I).
"""
import numpy as np
import pytest

from oracle import multislice as om

pytestmark = pytest.mark.gpu

N, D, NS, DZ, KEV, CS, DOSE = 2048, 0.1, 400, 0.5, 300.0, 1.0, 20.0
SLAB = 16


def _slab_atoms(seed=0):
    rng = np.random.default_rng(seed)
    n_atoms = int(round(0.1 * (N * D) ** 2 * NS * DZ))
    lo = np.array([-NS * DZ / 2, -N * D / 2, -N * D / 2])
    xyz = (lo + rng.random((n_atoms, 3)) * np.array([NS * DZ, N * D, N * D])).astype(np.float32)
    return xyz


def _fp64_pipeline(xyz, df, ap):
    """FP64 oracle: CUDA-rule binning, slice build and multislice in slabs of SLAB slices."""
    s, ins = om._cuda_axis_index(xyz[:, 0], NS, DZ)
    i1, in1 = om._cuda_axis_index(xyz[:, 1], N, D)
    i2, in2 = om._cuda_axis_index(xyz[:, 2], N, D)
    keep = ins & in1 & in2
    s, i1, i2 = s[keep], i1[keep], i2[keep]
    order = np.argsort(s, kind="stable")
    s, i1, i2 = s[order], i1[order], i2[order]
    bounds = np.searchsorted(s, np.arange(0, NS + SLAB, SLAB))
    sf = om.scattering_factors_half([6], N, N, D, D)
    wp = om.WavePropagator(N, N, D, D, KEV, "fftw", np.float64)
    psi = wp.init_wave(DOSE).astype(np.complex128)
    for k, s0 in enumerate(range(0, NS, SLAB)):
        a, b = bounds[k], bounds[k + 1]
        lin = (s[a:b] - s0) * N * N + i1[a:b] * N + i2[a:b]
        hist = np.bincount(lin, minlength=SLAB * N * N).astype(np.float64).reshape(1, SLAB, N, N)
        slices = om.make_slices(hist, sf, "fftw", np.float64)
        psi = wp.multislice_propagate(psi, slices, DZ)
    exit_wave = psi
    img = om.intensity(wp.lens_propagate(psi, CS, df, ap))
    return img, exit_wave


def test_precision_workload_2048x400():
    import torch

    import emsim_gb300.build as bld
    bld.build()
    from emsim_gb300 import backend, physics
    lam = physics.electron_wave_length_angstrom(KEV)
    df, ap = physics.scherzer_condition(lam, CS)
    xyz = _slab_atoms()
    b = backend.MultiSlicesBuilder([6], NS, N, N, DZ, D, D)
    slices = backend.build_slices_batch(b, [(xyz, [len(xyz)])])
    wp = backend.WavePropagator(N, N, D, D, KEV)
    img, ew = wp.image(slices[0], DZ, DOSE, CS, df, ap, return_exit_wave=True)
    img, ew = np.asarray(img.get()), np.asarray(ew.get())
    del slices
    torch.cuda.empty_cache()
    ref_img, ref_ew = _fp64_pipeline(xyz, df, ap)
    e_img = om.rel_l2(img, ref_img)
    e_ew = om.rel_l2(ew, ref_ew)
    e_con = om.rel_l2(img - img.mean(), ref_img - ref_img.mean())
    print(f"\nprecision 2048^2 x 400 slices, {len(xyz)} atoms: FP32 vs FP64 rel-L2 image {e_img:.3e}, "
          f"exit wave {e_ew:.3e}, contrast (I - mean) {e_con:.3e}")
    assert e_img < 1e-5
    assert e_ew < 1e-5
