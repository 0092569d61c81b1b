"""Import the reference emsim package (numpy backend, or its FFTW backend with the
extension built by ``oracle/ref_fftw/build.py``) from its source tree.

Test infrastructure only, and usable only where the reference tree exists (the
development container; never a GPU host).  Its location comes from the environment
variable ``EMSIM_REFERENCE_ROOT`` (the fixture-generating scripts under ``tests/golden``
set it).  Two shims are needed to import it
unchanged:

* ``emsim/utils/pdb.py:12-13`` imports Biopython at package import; Biopython is not
  installed, so empty ``Bio``/``Bio.PDB``/``Bio.PDB.MMCIF2Dict`` modules stand in (the
  PDB reader is never called here).
* ``emsim/__init__.py:24`` writes ``~/emsimConfig.ini`` at import; ``HOME`` is pointed
  at a temporary directory for the import.
"""
from __future__ import annotations

import os
import sys
import tempfile
import types
from pathlib import Path

def reference_root():
    v = os.environ.get("EMSIM_REFERENCE_ROOT")
    return Path(v) if v else None


def available() -> bool:
    root = reference_root()
    return root is not None and (root / "emsim" / "__init__.py").is_file()


def load():
    """Return the imported reference ``emsim`` package (numpy backend selected)."""
    if not available():
        raise RuntimeError(f"reference emsim tree not found (EMSIM_REFERENCE_ROOT={reference_root()})")
    REFERENCE_ROOT = reference_root()
    if "emsim" in sys.modules:
        return sys.modules["emsim"]
    sys.dont_write_bytecode = True
    for name in ("Bio", "Bio.PDB", "Bio.PDB.MMCIF2Dict"):
        sys.modules.setdefault(name, types.ModuleType(name))
    for attr in ("PDBList", "MMCIFParser", "PDBParser"):
        setattr(sys.modules["Bio.PDB"], attr, object)
    sys.modules["Bio.PDB.MMCIF2Dict"].MMCIF2Dict = object
    old_home = os.environ.get("HOME")
    os.environ["HOME"] = tempfile.mkdtemp(prefix="emsim_home_")
    sys.path.insert(0, str(REFERENCE_ROOT))
    try:
        import emsim  # noqa: F401
    finally:
        sys.path.remove(str(REFERENCE_ROOT))
        if old_home is not None:
            os.environ["HOME"] = old_home
    import logging
    logging.getLogger("emsim").setLevel(logging.WARNING)
    emsim.config.set_backend("numpy")
    return emsim


def load_fftw():
    """Return the reference ``emsim`` package with its FFTW backend selected: the
    extension modules ``wave_kernel`` / ``slice_kernel``, compiled from the reference's
    C++ by ``oracle.ref_fftw.build`` (built on first use), take the place of the
    package files ``emsim.backend.fftw_ext`` would hold."""
    import importlib.machinery
    import importlib.util

    em = load()
    from oracle.ref_fftw import build as rb
    mods = rb.built()
    if len(mods) < 2:
        mods = rb.build(reference_root())
    import emsim.backend.fftw_ext as ext
    for name, path in mods.items():
        full = f"emsim.backend.fftw_ext.{name}"
        if full not in sys.modules:
            loader = importlib.machinery.ExtensionFileLoader(full, str(path))
            spec = importlib.util.spec_from_file_location(full, str(path), loader=loader)
            mod = importlib.util.module_from_spec(spec)
            loader.exec_module(mod)
            sys.modules[full] = mod
        setattr(ext, name, sys.modules[full])
    em.config.set_backend("fftw")
    return em
