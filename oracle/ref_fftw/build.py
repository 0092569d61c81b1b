"""Build emsim's FFTW extension (``wave_kernel``, ``slice_kernel``) from the reference
source tree into ``oracle/_ref/``, against the oracle's own FFTW-interface transforms
(``fftw3.h``, ``fftw_stub.cpp`` here) in place of libfftw3f, which is not installed.

The reference's C++ (``emsim/backend/fftw_ext/src/{WavePropagator,SliceBuilder}.cpp``)
and its pybind11 bindings (``wave_kernel.cpp``, ``slice_kernel.cpp``) are compiled where
they lie, unchanged, with g++ -fopenmp; only the transforms are the oracle's.  Checker
infrastructure: it runs only where the reference tree exists (never on a GPU host) and
its outputs stay out of the repository.  The reference's own build (CMake with
find_package(FFTW)) is not used.

Usage:  python -m oracle.ref_fftw.build [REFERENCE_ROOT]
"""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE.parent / "_ref"


DEFAULT_ROOT = "/root/reference"


def reference_src(root=None) -> Path:
    root = Path(root or os.environ.get("EMSIM_REFERENCE_ROOT") or DEFAULT_ROOT)
    return root / "emsim" / "backend" / "fftw_ext" / "src"


def build_if_available(root=None) -> dict:
    """build() where the reference tree exists; nothing (an empty dict) elsewhere."""
    if not (reference_src(root) / "WavePropagator.cpp").is_file():
        return {}
    return build(root)


def built() -> dict:
    """Paths of the built modules that exist (empty where they were not built)."""
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    out = {}
    for name in ("wave_kernel", "slice_kernel"):
        p = OUT / f"{name}{suffix}"
        if p.is_file():
            out[name] = p
    return out


def build(root=None, force: bool = False) -> dict:
    src = reference_src(root)
    if not (src / "WavePropagator.cpp").is_file():
        raise FileNotFoundError(f"reference FFTW extension sources not found under {src}")
    try:
        import pybind11
    except ImportError as e:  # pragma: no cover - pybind11 is in the development image
        raise RuntimeError("pybind11 is needed to build the reference bindings") from e
    OUT.mkdir(parents=True, exist_ok=True)
    suffix = sysconfig.get_config_var("EXT_SUFFIX")
    inc = ["-I", str(HERE), "-I", str(src), "-I", pybind11.get_include(), "-I", sysconfig.get_paths()["include"]]
    flags = ["-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-fvisibility=hidden"]
    jobs = {"wave_kernel": ["WavePropagator.cpp", "wave_kernel.cpp"],
            "slice_kernel": ["SliceBuilder.cpp", "slice_kernel.cpp"]}
    procs = []
    for name, files in jobs.items():
        target = OUT / f"{name}{suffix}"
        if target.is_file() and not force:
            continue
        cmd = ["g++", *flags, *inc, *[str(src / f) for f in files], str(HERE / "fftw_stub.cpp"), "-o", str(target)]
        procs.append((name, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)))
    for name, p in procs:
        _, err = p.communicate()
        if p.returncode != 0:
            raise RuntimeError(f"building the reference {name} failed:\n{err}")
    return built()


if __name__ == "__main__":
    print(build(sys.argv[1] if len(sys.argv) > 1 else None, force=True))
