"""Record the backend calls that emsim's own front-end makes, as a replayable fixture.

emsim's front-end (``emsim.pot``, ``emsim.wave``, ``emsim.tem``, ``emsim.pipe``) resolves
its three backend classes from ``emsim.config.get_current_backend()`` at every call.
This script imports the reference package from its source tree (``oracle/ref_numpy.py``),
puts a recording backend in front of its numpy backend, and runs the front-end the way
its demo and pipeline do:

* five atoms (Z = 6, 14, 29, 79, 92 along y at 5..45 A, centralized), 512^2 at pixel
  50/512 A, 200 keV, Cs 1.3 mm, Scherzer: ``pot.build_one_slice`` ->
  ``TEM.get_wave_propagator`` -> ``init_wave`` -> ``slice_transmit`` -> ``lens_propagate``
  (demos/five_atoms.py);
* ``pipe.Pipe(...).run`` of a 3000-atom C/N/O/S blob at roi 64, resolution 1 A, 2 A
  slices, 200 keV, Cs 1.3 mm, defocus 700 A, aperture 10 mrad, no water (pipe.py:79-84).

Every constructor and method call reaching the backend is written down with its
arguments: arrays produced by the front-end (coordinates, element lists, counts) are
stored, arrays returned by an earlier backend call are stored as references to that
call, scalars as they came.  A small centre crop of each scenario's final output (the
reference numpy backend's) is stored too.  ``tests/test_host_logic.py`` checks that
every recorded call binds to the GB300 backend's signatures; ``tests/test_gpu_frontend.py``
replays the calls through the GB300 backend on a GPU.

Usage:  python tests/golden/make_frontend_trace.py
"""
from __future__ import annotations

import json
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))
os.environ.setdefault("EMSIM_REFERENCE_ROOT", "/root/reference")

from oracle import ref_numpy  # noqa: E402

CROP = 32  # side of the stored centre crop of each scenario's output


class Recorder:
    def __init__(self):
        self.records = []
        self.arrays = {}
        self.results = {}  # id(result object) -> call index
        self.keep = []     # keeps recorded results alive so their ids stay unique
        self.n_objects = 0

    def enc(self, x):
        if isinstance(x, np.ndarray):
            if id(x) in self.results:
                return {"ref": self.results[id(x)]}
            key = f"a{len(self.arrays)}"
            self.arrays[key] = x
            return {"array": key}
        if isinstance(x, (tuple, list)):
            return {"seq": [self.enc(v) for v in x], "tuple": isinstance(x, tuple)}
        if isinstance(x, (np.integer,)):
            return {"int": int(x)}
        if isinstance(x, (np.floating,)):
            return {"float": float(x)}
        if isinstance(x, bool) or x is None:
            return {"value": x}
        if isinstance(x, int):
            return {"int": x}
        if isinstance(x, float):
            return {"float": x}
        raise TypeError(f"cannot record argument of type {type(x)}")

    def wrap(self, name, cls):
        rec = self

        class Recorded:
            def __init__(self, *args, **kwargs):
                self._inner = cls(*args, **kwargs)
                self._oid = rec.n_objects
                rec.n_objects += 1
                rec.records.append({"op": "new", "cls": name, "oid": self._oid, "args": [rec.enc(a) for a in args],
                                    "kwargs": {k: rec.enc(v) for k, v in kwargs.items()}})

            def __getattr__(self, attr):
                f = getattr(self._inner, attr)
                if not callable(f):
                    return f

                def call(*args, **kwargs):
                    entry = {"op": "call", "oid": self._oid, "cls": name, "method": attr,
                             "args": [rec.enc(a) for a in args], "kwargs": {k: rec.enc(v) for k, v in kwargs.items()}}
                    out = f(*args, **kwargs)
                    entry["index"] = len(rec.records)
                    rec.records.append(entry)
                    if isinstance(out, np.ndarray):
                        rec.results[id(out)] = entry["index"]
                        rec.keep.append(out)
                        entry["result_shape"] = list(out.shape)
                        entry["result_dtype"] = str(out.dtype)
                    return out
                return call

        Recorded.__name__ = name
        return Recorded


class RecordingBackend:
    """A stand-in for emsim.config.Backend: the numpy backend's classes behind recorders."""

    def __init__(self, rec, numpy_backend):
        self.one_slice_builder = rec.wrap("OneSliceBuilder", numpy_backend.one_slice_builder)
        self.multi_slices_builder = rec.wrap("MultiSlicesBuilder", numpy_backend.multi_slices_builder)
        self.wave_propagator = rec.wrap("WavePropagator", numpy_backend.wave_propagator)


def crop(a):
    n1, n2 = a.shape[-2:]
    return np.ascontiguousarray(a[..., n1 // 2 - CROP // 2:n1 // 2 + CROP // 2, n2 // 2 - CROP // 2:n2 // 2 + CROP // 2])


def main():
    em = ref_numpy.load()
    from oracle import multislice as om
    em.config.set_backend("numpy")
    rec = Recorder()
    em.config._current_backend = RecordingBackend(rec, em.config.get_current_backend())
    scenarios = []

    # five atoms, demos/five_atoms.py (with int64 elements: the demo's np.int is gone from numpy)
    t = em.tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10.37e-3)
    t.set_scherzer_condition()
    mol = em.atoms.AtomList(elements=np.array([6, 14, 29, 79, 92], dtype=np.int64),
                            coordinates=np.array([[0, 0, 5], [0, 0, 15], [0, 0, 25], [0, 0, 35], [0, 0, 45]],
                                                 dtype=np.float32))
    mol = em.atoms.centralize(mol)
    first = len(rec.records)
    propagator = t.get_wave_propagator(wave_shape=(512, 512), pixel_size=50 / 512)
    aslice = em.pot.build_one_slice(mol, pixel_size=50 / 512, lateral_size=(512, 512))
    wave = propagator.init_wave()
    exit_wave = propagator.slice_transmit(wave, aslice)
    image_wave = propagator.lens_propagate(exit_wave)
    image = np.abs(image_wave) ** 2
    scenarios.append({"name": "five_atoms_512", "first": first, "last": len(rec.records),
                      "output": rec.results[id(image_wave)], "final": "intensity"})
    out = {"five_atoms_512_crop": crop(image)}

    # Pipe.run of a small blob
    el, xyz = om.protein_blob(3000, radius=15.0, seed=21)
    t2 = em.tem.TEM(electron_dose=20, beam_energy_kev=200, cs_mm=1.3, defocus=700, aperture=10e-3)
    p = em.pipe.Pipe(t2, resolution=1.0, slice_thickness=2.0, roi=64, add_water=False)
    first = len(rec.records)
    img = p.run(em.atoms.AtomList(elements=el, coordinates=xyz))
    # the Pipe computes |psi|^2 of the lens_propagate result itself (pipe.py:79-84)
    lens_calls = [r for r in rec.records[first:] if r.get("method") == "lens_propagate"]
    scenarios.append({"name": "pipe_run_blob_64", "first": first, "last": len(rec.records),
                      "output": lens_calls[-1]["index"], "final": "intensity"})
    out["pipe_run_blob_64_crop"] = crop(img)

    trace = {"records": rec.records, "scenarios": scenarios, "crop": CROP,
             "reference": "emsim front-end with the numpy backend (emsim/pot.py, emsim/wave.py, emsim/tem.py, "
                          "emsim/pipe.py)"}
    arrays = {k: v for k, v in rec.arrays.items()}
    arrays.update(out)
    arrays["trace_json"] = np.frombuffer(json.dumps(trace).encode(), dtype=np.uint8)
    np.savez_compressed(HERE / "golden_frontend_trace.npz", **arrays)
    print(f"{len(rec.records)} backend calls, {len(rec.arrays)} input arrays, "
          f"{(HERE / 'golden_frontend_trace.npz').stat().st_size} bytes")


if __name__ == "__main__":
    main()
