"""Generate golden vectors by running the reference emsim numpy path on seeded inputs.

Runs only where the reference source tree exists (see ``oracle/ref_numpy.py``); the
resulting ``*.npz`` fixtures are committed and read by the tests everywhere else.
Every fixture stores its inputs next to the reference outputs, so no test needs the
random generator to reproduce them.

Usage:  python tests/golden/make_golden.py [generator ...]
"""
from __future__ import annotations

import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
os.environ.setdefault("EMSIM_REFERENCE_ROOT", "/root/reference")

from oracle import ref_numpy  # noqa: E402


def _atoms_in_box(rng, n, half_extent, elements=(1, 6, 7, 8, 16, 29)):
    el = rng.choice(np.array(elements), size=n)
    xyz = (rng.random((n, 3)) * 2 - 1) * np.asarray(half_extent)
    return el, xyz.astype(np.float32)


def physics(em):
    kev = np.array([60., 80., 120., 200., 300.])
    ph = em.physics
    out = dict(
        kev=kev,
        wave_length=np.array([ph.electron_wave_length_angstrom(k) for k in kev]),
        gamma=np.array([ph.electron_relativity_gamma(k) for k in kev]),
        sigma=np.array([ph.interaction_parameter(k) for k in kev]),
    )
    sch = []
    for k, cs in [(200., 1.3), (300., 1.0), (120., 2.0)]:
        sch.append((k, cs) + tuple(ph.scherzer_condition(ph.electron_wave_length_angstrom(k), cs)))
    out["scherzer"] = np.array(sch)
    np.savez_compressed(HERE / "golden_physics.npz", **out)


def scattering(em):
    zs = [1, 6, 7, 8, 16, 29, 79, 92]
    out = {"zs": np.array(zs)}
    from emsim.backend.slice_builder_base import OneSliceBuilderBase
    for tag, (n1, n2, d1, d2) in {"a": (32, 32, 0.5, 0.5), "b": (24, 40, 0.3, 0.45),
                                  "c": (33, 31, 0.2, 0.25)}.items():
        out[f"grid_{tag}"] = np.array([n1, n2, d1, d2])
        out[f"sf2d_{tag}"] = em.elem.scattering_factors2d(zs, n1, n2, d1, d2)
        out[f"half_{tag}"] = OneSliceBuilderBase(zs, n1, n2, d1, d2).scattering_factors
    np.savez_compressed(HERE / "golden_scattering.npz", **out)


def binning(em):
    from emsim.backend import slice_builder_base as sbb
    rng = np.random.default_rng(1234)
    out = {}
    cases = {
        # (shape, steps)
        "one_even": ((24, 30), (0.5, 0.4)),
        "one_odd": ((25, 31), (0.5, 0.4)),
        "multi_even": ((6, 16, 20), (1.3, 0.5, 0.45)),
        "multi_odd": ((7, 17, 21), (1.3, 0.5, 0.45)),
    }
    for tag, (shape, steps) in cases.items():
        full = [0.0] * (3 - len(shape)) + [s * d / 2 * 1.1 for s, d in zip(shape, steps)]
        el, xyz = _atoms_in_box(rng, 600, full if len(shape) == 3 else [1.0] + full[1:])
        # atoms exactly on the numpy-rule edges (first and last edge of each axis)
        edge = []
        axes = (1, 2) if len(shape) == 2 else (0, 1, 2)
        for ax, n, d in zip(axes, shape, steps):
            start = -d * (n // 2)
            for v in (start, start + n * d, 0.0):
                p = np.zeros(3, np.float32)
                p[ax] = v
                edge.append(p)
        xyz = np.concatenate([xyz, np.array(edge, np.float32)])
        el = np.concatenate([el, np.full(len(edge), 6)])
        mol = em.atoms.AtomList(elements=el, coordinates=xyz)
        mol, uz, cnt = em.atoms.sort_elements_and_count(mol)
        if len(shape) == 2:
            h = sbb._bin_atoms_one_slice(mol.coordinates, cnt, *shape, *steps)
        else:
            h = sbb._bin_atoms_multi_slices(mol.coordinates, cnt, *shape, *steps)
        out[f"{tag}_coords"] = mol.coordinates
        out[f"{tag}_elements"] = mol.elements
        out[f"{tag}_uz"] = uz
        out[f"{tag}_counts"] = cnt
        out[f"{tag}_shape"] = np.array(shape)
        out[f"{tag}_steps"] = np.array(steps)
        out[f"{tag}_hist"] = h
    np.savez_compressed(HERE / "golden_binning.npz", **out)


def slices(em):
    from emsim.backend import slice_builder_numpy as sbn
    rng = np.random.default_rng(99)
    out = {}
    # direct builder calls on seeded histograms
    zs = [6, 7, 8, 16]
    n1, n2, d1, d2, ns, dz = 32, 32, 0.5, 0.5, 3, 2.0
    hist = rng.poisson(0.05, size=(len(zs), ns, n1, n2)).astype(np.float32)
    msb = sbn.MultiSlicesBuilder(zs, ns, n1, n2, dz, d1, d2)
    out.update(ms_zs=np.array(zs), ms_grid=np.array([ns, n1, n2, dz, d1, d2]), ms_hist=hist,
               ms_sf=msb.scattering_factors, ms_slices=msb.make_multi_slices(hist.copy()))
    osb = sbn.OneSliceBuilder(zs, n1, n2, d1, d2)
    out.update(os_hist=hist[:, 0].copy(), os_slice=osb.make_one_slice(hist[:, 0].copy()))
    # front-end: five atoms, one slice at 48^2
    el = np.array([6, 14, 29, 79, 92])
    xyz = np.array([[0, 0, 5], [0, 0, 15], [0, 0, 25], [0, 0, 35], [0, 0, 45]], dtype=np.float32)
    mol = em.atoms.centralize(em.atoms.AtomList(elements=el, coordinates=xyz))
    out.update(five_coords=mol.coordinates, five_elements=el,
               five_slice=em.pot.build_one_slice(mol, pixel_size=50 / 48, lateral_size=(48, 48)))
    # front-end: small blob, multi slice, size from the extent
    el, xyz = _atoms_in_box(rng, 300, [6.0, 7.0, 7.0], elements=(6, 7, 8, 16))
    mol = em.atoms.centralize(em.atoms.AtomList(elements=el, coordinates=xyz))
    out.update(blob_coords=mol.coordinates, blob_elements=el,
               blob_slices=em.pot.build_multi_slices(mol, dz=2.0, pixel_size=1.0, lateral_size=16))
    np.savez_compressed(HERE / "golden_slices.npz", **out)


def waves(em):
    from emsim.backend import wave_propagator_numpy as wpn
    rng = np.random.default_rng(7)
    out = {}
    for tag, (n1, n2, d) in {"sq": (32, 32, 0.4), "rect": (24, 40, 0.5)}.items():
        wp = wpn.WavePropagator(n1, n2, d, d, 200.0)
        w = (rng.normal(size=(n1, n2)) + 1j * rng.normal(size=(n1, n2))).astype(np.complex64)
        sl = np.abs(rng.normal(size=(3, n1, n2))) * 2.0
        lam = em.physics.electron_wave_length_angstrom(200.0)
        df, ap = em.physics.scherzer_condition(lam, 1.3)
        out.update({
            f"{tag}_grid": np.array([n1, n2, d]), f"{tag}_wave": w, f"{tag}_slices": sl,
            f"{tag}_init": wp.init_wave(20.0),
            f"{tag}_transmit": wp.slice_transmit(w, sl[0]),
            f"{tag}_space": wp.space_propagate(w, 2.0),
            f"{tag}_single": wp.singleslice_propagate(w, sl[0], 2.0),
            f"{tag}_multi": wp.multislice_propagate(w, sl, 2.0),
            f"{tag}_lens": wp.lens_propagate(w, 1.3, df, ap),
            f"{tag}_lens_params": np.array([1.3, df, ap]),
        })
    np.savez_compressed(HERE / "golden_wave.npz", **out)


def pipes(em):
    rng = np.random.default_rng(2024)
    el, xyz = _atoms_in_box(rng, 400, [8.0, 9.0, 9.0], elements=(6, 7, 8, 16))
    mol = em.atoms.AtomList(elements=el, coordinates=xyz)
    tem = em.tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    p = em.pipe.Pipe(tem, resolution=2.0, slice_thickness=2.0, roi=32, add_water=False)
    img = p.run(mol)
    # five atoms, 128^2, one slice through transmit and lens (Scherzer)
    tem5 = em.tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10.37e-3)
    tem5.set_scherzer_condition()
    el5 = np.array([6, 14, 29, 79, 92])
    xyz5 = np.array([[0, 0, 5], [0, 0, 15], [0, 0, 25], [0, 0, 35], [0, 0, 45]], dtype=np.float32)
    mol5 = em.atoms.centralize(em.atoms.AtomList(elements=el5, coordinates=xyz5))
    prop = tem5.get_wave_propagator(wave_shape=(128, 128), pixel_size=50 / 128)
    aslice = em.pot.build_one_slice(mol5, pixel_size=50 / 128, lateral_size=(128, 128))
    ew = prop.slice_transmit(prop.init_wave(), aslice)
    iw = prop.lens_propagate(ew)
    np.savez_compressed(HERE / "golden_pipe.npz", blob_elements=el, blob_coords=xyz, blob_image=img,
                        five_slice=aslice, five_exit=ew, five_image=np.abs(iw) ** 2,
                        five_tem=np.array([tem5.defocus, tem5.aperture]))


def specimen(em):
    """tem.band_limit_specimen on a cubic stack, the one shape for which the reference's
    axes (0, 1) transform and its fil[..., None] broadcast agree (tem.py:102-108)."""
    rng = np.random.default_rng(41)
    x = rng.random((16, 16, 16)) * 10.0
    out = em.tem.band_limit_specimen(em.tem.Specimen(x, 1.0, 2.0)).slices
    np.savez_compressed(HERE / "golden_specimen.npz", cube=x, band_limited=out)


GENERATORS = {"physics": physics, "scattering": scattering, "binning": binning, "slices": slices,
              "waves": waves, "pipes": pipes, "specimen": specimen}


def main(names=None):
    """Regenerate every fixture, or only the named ones."""
    em = ref_numpy.load()
    for name in names or list(GENERATORS):
        GENERATORS[name](em)
    for f in sorted(HERE.glob("golden_*.npz")):
        print(f.name, f.stat().st_size)


if __name__ == "__main__":
    main(sys.argv[1:])
