"""emsim_gb300 - GB300 (sm_103a) multislice engine behind emsim's Python API.

Modules mirror emsim's: ``atoms``, ``elem``, ``physics``, ``pot``, ``wave``, ``tem``,
``pipe``, ``simulator``; ``backend`` holds the three plugin classes and ``config.register``
makes ``emsim.config.set_backend("gb300")`` select them.  All numerics run in the
compiled library ``_lib/libemsim_gb300.so`` (C ABI: ``include/emsim_gb300.h``).
"""
from . import atoms, config, elem, physics  # noqa: F401

__all__ = ["atoms", "config", "elem", "physics", "backend", "pot", "wave", "tem", "pipe", "simulator"]


def __getattr__(name):
    # device-side modules import torch lazily
    if name in ("backend", "pot", "wave", "tem", "pipe", "simulator"):
        import importlib
        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)
