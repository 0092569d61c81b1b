"""Replay of the backend calls recorded from emsim's own front-end
(tests/golden/make_frontend_trace.py) against any backend module that provides
``OneSliceBuilder``, ``MultiSlicesBuilder`` and ``WavePropagator``."""
from __future__ import annotations

import json
from pathlib import Path

import numpy as np

FIXTURE = Path(__file__).resolve().parent / "golden" / "golden_frontend_trace.npz"


def load():
    d = np.load(FIXTURE)
    trace = json.loads(bytes(d["trace_json"]).decode())
    return trace, d


def decode(x, arrays, results, as_array=lambda a: a):
    if "ref" in x:
        return results[x["ref"]]
    if "array" in x:
        return as_array(arrays[x["array"]])
    if "seq" in x:
        seq = [decode(v, arrays, results, as_array) for v in x["seq"]]
        return tuple(seq) if x["tuple"] else seq
    if "int" in x:
        return int(x["int"])
    if "float" in x:
        return float(x["float"])
    return x["value"]


def replay(backend, records, arrays, as_array=lambda a: a):
    """Run every recorded call on ``backend``; returns {call index: result}."""
    objs, results = {}, {}
    for r in records:
        args = [decode(a, arrays, results, as_array) for a in r["args"]]
        kwargs = {k: decode(v, arrays, results, as_array) for k, v in r["kwargs"].items()}
        if r["op"] == "new":
            objs[r["oid"]] = getattr(backend, r["cls"])(*args, **kwargs)
        else:
            results[r["index"]] = getattr(objs[r["oid"]], r["method"])(*args, **kwargs)
    return results


def oracle_backend(semantics: str = "fftw", dtype=np.float64):
    """The oracle's restatement behind the backend classes' interface (CPU)."""
    from oracle import multislice as om

    class OneSliceBuilder:
        def __init__(self, unique_elements, n1, n2, d1, d2):
            self.n1, self.n2, self.d1, self.d2 = n1, n2, d1, d2
            self.sf = om.scattering_factors_half(list(unique_elements), n1, n2, d1, d2)

        def bin_atoms_one_slice(self, coords, counts):
            b = om.bin_atoms_numpy if semantics == "numpy" else om.bin_atoms_cuda
            return b(coords, counts, (self.n1, self.n2), (self.d1, self.d2))

        def make_one_slice(self, hist, symmetric_bandlimit=True):
            return om.make_slices(hist, self.sf, semantics, dtype, symmetric_bandlimit)

    class MultiSlicesBuilder:
        def __init__(self, unique_elements, n_slices, n1, n2, dz, d1, d2):
            self.shape, self.steps = (n_slices, n1, n2), (dz, d1, d2)
            self.sf = om.scattering_factors_half(list(unique_elements), n1, n2, d1, d2)

        def bin_atoms_multi_slices(self, coords, counts):
            b = om.bin_atoms_numpy if semantics == "numpy" else om.bin_atoms_cuda
            return b(coords, counts, self.shape, self.steps)

        def make_multi_slices(self, hist, symmetric_bandlimit=True):
            return om.make_slices(hist, self.sf, semantics, dtype, symmetric_bandlimit)

    class WavePropagator(om.WavePropagator):
        def __init__(self, n1, n2, d1, d2, beam_energy_kev):
            super().__init__(n1, n2, d1, d2, beam_energy_kev, semantics, dtype)

    class Backend:
        pass

    Backend.OneSliceBuilder = OneSliceBuilder
    Backend.MultiSlicesBuilder = MultiSlicesBuilder
    Backend.WavePropagator = WavePropagator
    return Backend


def crop(a, side):
    n1, n2 = a.shape[-2:]
    return a[..., n1 // 2 - side // 2:n1 // 2 + side // 2, n2 // 2 - side // 2:n2 // 2 + side // 2]
