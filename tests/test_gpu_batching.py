"""The batching workload through the product API, against the FP64 oracle.

Eight blobs of the batching mix (synth.batching_mix, seed 11): C/N/O/S at 0.1 A^-3 with
log-uniform atom counts, each in a uniform random orientation, roi 256 or 512 at pixel
1 A, every odd-numbered one embedded in amorphous ice (O at 0.0334 A^-3 plus two H per O
within 1 A, over the field of view).  All eight go through one Pipe.run_batch call (a
ragged batch: two lateral sizes on their own streams, each molecule on its own slice
count); the images of an iced 512^2 blob (1.25 M atoms), an iced 256^2 blob and a plain
256^2 blob are compared with the oracle's FP64 restatement of the reference's native
semantics, relative L2 <= 1e-5.
"""
import numpy as np
import pytest

from oracle import multislice as om

pytestmark = pytest.mark.gpu

TOL = 1e-5
CHECK = [0, 3, 5]  # plain 256^2, iced 512^2, iced 256^2


def test_batching_mix_run_batch_against_fp64():
    import emsim_gb300.build as b
    b.build()
    from emsim_gb300 import atoms, pipe, synth, tem
    mix = synth.batching_mix(8, seed=11, pixel=1.0)
    assert [mix[k][2] for k in CHECK] == [256, 512, 256]
    assert all(1 in set(mix[k][0].tolist()) for k in (3, 5))
    t = tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    p = pipe.Pipe(t, resolution=2.0, slice_thickness=2.0, roi=256, add_water=False)
    mols = [atoms.AtomList(el, xyz) for el, xyz, _ in mix]
    rois = [r for _, _, r in mix]
    imgs = p.run_batch(mols, rois=rois, to_host=True)
    assert [im.shape[0] for im in imgs] == rois
    for k in CHECK:
        el, xyz, roi = mix[k]
        ref = om.pipe_run(el, xyz, resolution=2.0, slice_thickness=2.0, roi=roi, beam_energy_kev=200, dose=20,
                          cs_mm=1.3, defocus=700, aperture=10e-3, semantics="fftw", dtype=np.float64)
        err = om.rel_l2(imgs[k], ref)
        con = om.rel_l2(imgs[k] - imgs[k].mean(), ref - ref.mean())
        print(f"\nblob {k}: {len(el)} atoms, roi {roi}: rel-L2 vs FP64 {err:.3e} (contrast {con:.3e})")
        assert err < TOL, (k, err)
