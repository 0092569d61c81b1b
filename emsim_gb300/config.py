"""Backend registration.

emsim selects backends with ``emsim.config.set_backend(name)`` and resolves the three
plugin classes from ``config.get_current_backend()`` at each call
(emsim/config.py:10-69, pot.py:16,38, wave.py:14-15).  ``register(emsim)`` extends an
imported emsim package so that ``set_backend("gb300")`` selects this engine; every
other name keeps its original behaviour.
"""
from __future__ import annotations

import types


class Gb300Backend:
    backend_type = "gb300"

    @property
    def one_slice_builder(self):
        from . import backend
        return backend.OneSliceBuilder

    @property
    def multi_slices_builder(self):
        from . import backend
        return backend.MultiSlicesBuilder

    @property
    def wave_propagator(self):
        from . import backend
        return backend.WavePropagator

    def __repr__(self):
        return "<emsim backend gb300>"


def register(emsim_module: types.ModuleType) -> None:
    cfg = emsim_module.config
    if getattr(cfg, "_gb300_registered", False):
        return
    original = cfg.set_backend

    def set_backend(backend="numpy"):
        if isinstance(backend, str) and backend.lower() == "gb300":
            cfg._current_backend = Gb300Backend()
            return
        original(backend)

    cfg.set_backend = set_backend
    cfg._gb300_registered = True
