"""Import the reference emsim package (numpy backend) from its source tree.

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
