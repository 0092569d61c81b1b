"""ctypes binding of the engine's C ABI (``include/emsim_gb300.h``).

The shared library is built in-tree by ``emsim_gb300.build``.  There is no fallback:
when the library is missing or fails to load, every entry point raises
:class:`NativeUnavailable`.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libemsim_gb300.so"

_c_int, _c_ll, _c_dbl, _c_uint, _c_vp = ctypes.c_int, ctypes.c_longlong, ctypes.c_double, ctypes.c_uint, ctypes.c_void_p
_c_size = ctypes.c_size_t
_c_dbl_p = ctypes.POINTER(ctypes.c_double)
_pp = ctypes.POINTER(ctypes.c_void_p)

# name -> (restype, argtypes); mirrors include/emsim_gb300.h one to one
SIGNATURES = {
    "emsim_gb300_abi_version": (_c_int, []),
    "emsim_gb300_last_error": (ctypes.c_char_p, []),
    "emsim_gb300_check_device_error": (_c_int, [ctypes.POINTER(ctypes.c_int)]),
    "emsim_gb300_peek_device_error": (_c_int, [ctypes.POINTER(ctypes.c_int)]),
    "emsim_gb300_set_wait_limit_ns": (_c_int, [ctypes.c_ulonglong]),
    "emsim_gb300_get_wait_limit_ns": (ctypes.c_ulonglong, []),
    "emsim_gb300_wait_timeout_probe": (_c_int, [ctypes.c_ulonglong, _c_vp, _c_vp]),
    "emsim_gb300_wave_plan_create": (_c_int, [_c_int, _c_int, _c_dbl, _c_dbl, _c_dbl, _c_dbl, _pp]),
    "emsim_gb300_wave_plan_destroy": (_c_int, [_c_vp]),
    "emsim_gb300_init_wave": (_c_int, [_c_vp, _c_dbl, _c_vp, _c_int, _c_vp]),
    "emsim_gb300_slice_transmit": (_c_int, [_c_vp, _c_vp, _c_vp, _c_ll, _c_vp, _c_int, _c_vp]),
    "emsim_gb300_space_propagate": (_c_int, [_c_vp, _c_vp, _c_dbl, _c_vp, _c_int, _c_vp]),
    "emsim_gb300_singleslice_propagate": (_c_int, [_c_vp, _c_vp, _c_vp, _c_ll, _c_dbl, _c_vp, _c_int, _c_vp]),
    "emsim_gb300_multislice_propagate": (_c_int, [_c_vp, _c_vp, _c_vp, _c_int, _c_ll, _c_dbl, _c_vp, _c_int, _c_vp]),
    "emsim_gb300_lens_propagate": (_c_int, [_c_vp, _c_vp, _c_dbl, _c_dbl, _c_dbl, _c_vp, _c_int, _c_vp]),
    "emsim_gb300_lens_incoherent_workspace_size": (_c_size, [_c_vp, _c_int]),
    "emsim_gb300_lens_intensity_incoherent": (_c_int, [_c_vp, _c_vp, _c_int, _c_dbl, _c_dbl_p, _c_dbl_p, _c_int,
                                                       _c_dbl, _c_dbl, _c_vp, _c_vp, _c_size, _c_vp]),
    "emsim_gb300_intensity": (_c_int, [_c_vp, _c_vp, _c_ll, _c_vp]),
    "emsim_gb300_multislice_image": (_c_int, [_c_vp, _c_vp, _c_int, _c_ll, _c_dbl, _c_dbl, _c_dbl,
                                              ctypes.POINTER(ctypes.c_double), _c_int, _c_dbl, _c_vp, _c_vp,
                                              _c_vp, _c_int, _c_vp]),
    "emsim_gb300_slice_plan_create": (_c_int, [_c_vp, _c_int, _c_int, _c_int, _c_int, _c_dbl, _c_dbl, _c_dbl,
                                               _c_int, _pp]),
    "emsim_gb300_slice_plan_destroy": (_c_int, [_c_vp]),
    "emsim_gb300_bin_atoms_one_slice": (_c_int, [_c_vp, _c_vp, _c_uint, _c_vp, _c_vp, _c_vp]),
    "emsim_gb300_bin_atoms_multi_slices": (_c_int, [_c_vp, _c_vp, _c_uint, _c_vp, _c_vp, _c_vp]),
    "emsim_gb300_make_slices_workspace_size": (_c_size, [_c_vp]),
    "emsim_gb300_make_slices": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_size, _c_vp]),
    "emsim_gb300_build_slices_workspace_size": (_c_size, [_c_vp, _c_uint, _c_int]),
    "emsim_gb300_build_slices": (_c_int, [_c_vp, _c_vp, _c_uint, _c_vp, _c_int, _c_vp, _c_vp, _c_size, _c_vp]),
    "emsim_gb300_make_slices_noalloc": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp]),
    "emsim_gb300_band_limit_workspace_size": (_c_size, [_c_int, _c_int, _c_int]),
    "emsim_gb300_band_limit_slices": (_c_int, [_c_vp, _c_int, _c_int, _c_int, _c_vp, _c_vp, _c_size, _c_vp]),
    "emsim_gb300_add_water": (_c_int, [_c_vp, _c_vp, _c_int, _c_int, _c_dbl, ctypes.c_uint64, ctypes.c_uint32, _c_vp]),
    "emsim_gb300_centralize": (_c_int, [_c_vp, _c_vp, _c_vp, _c_int, _c_vp, _c_vp, _c_vp, _c_vp]),
    "emsim_gb300_build_slices_z": (_c_int, [_c_vp, _c_vp, _c_vp, _c_uint, _c_vp, _c_int, _c_vp, _c_vp, _c_vp, _c_int,
                                            _c_vp, _c_vp, _c_size, _c_vp]),
    "emsim_gb300_image_from_atoms_workspace_size": (_c_size, [_c_vp, _c_uint, _c_int, _c_int]),
    "emsim_gb300_image_from_atoms_z": (_c_int, [_c_vp, _c_vp, _c_vp, _c_vp, _c_uint, _c_vp, _c_int, _c_vp, _c_vp, _c_vp,
                                                _c_int, _c_dbl, _c_dbl, ctypes.POINTER(ctypes.c_double), _c_int,
                                                _c_dbl, _c_vp, _c_int, _c_vp, _c_size, _c_vp]),
    "emsim_gb300_smooth_workspace_size": (_c_size, [_c_vp, _c_uint, _c_int]),
    "emsim_gb300_build_slices_smooth": (_c_int, [_c_vp, _c_vp, _c_uint, _c_vp, _c_int, _c_vp, _c_vp, _c_size, _c_vp]),
    "emsim_gb300_build_slices_smooth_adjoint": (_c_int, [_c_vp, _c_vp, _c_uint, _c_vp, _c_int, _c_vp, _c_vp, _c_vp,
                                                         _c_vp, _c_size, _c_vp]),
    "emsim_gb300_set_precision": (_c_int, [_c_int]),
    "emsim_gb300_get_precision": (_c_int, []),
    "emsim_gb300_set_pass_tuning": (_c_int, [_c_int, _c_int, _c_int, _c_int, _c_int]),
    "emsim_gb300_get_pass_tuning": (_c_int, [_c_int, ctypes.POINTER(ctypes.c_int)]),
    "emsim_gb300_build_slices_ragged": (_c_int, [_c_vp, _c_vp, _c_vp, _c_uint, _c_vp, _c_int, _c_vp, _c_vp, _c_vp,
                                                 _c_vp, _c_int, _c_vp, _c_vp, _c_size, _c_vp]),
    "emsim_gb300_multislice_image_ragged": (_c_int, [_c_vp, _c_vp, _c_ll, ctypes.POINTER(ctypes.c_int32), _c_dbl,
                                                     _c_dbl, _c_dbl, ctypes.POINTER(ctypes.c_double), _c_int, _c_dbl,
                                                     _c_vp, _c_vp, _c_int, _c_vp]),
    "emsim_gb300_adjoint_checkpoints": (_c_int, [_c_int, _c_int]),
    "emsim_gb300_adjoint_workspace_size": (_c_size, [_c_vp, _c_int, _c_int, _c_int, _c_ll]),
    "emsim_gb300_multislice_image_ckpt": (_c_int, [_c_vp, _c_vp, _c_int, _c_ll, _c_dbl, _c_dbl, _c_dbl,
                                                   ctypes.POINTER(ctypes.c_double), _c_int, _c_dbl, _c_vp, _c_vp,
                                                   _c_vp, _c_int, _c_int, _c_vp]),
    "emsim_gb300_multislice_image_adjoint": (_c_int, [_c_vp, _c_vp, _c_int, _c_ll, _c_dbl, _c_dbl, _c_dbl,
                                                      ctypes.POINTER(ctypes.c_double), _c_int, _c_dbl, _c_vp, _c_vp,
                                                      _c_vp, _c_int, _c_vp, _c_vp, _c_size, _c_int, _c_vp]),
}

ERROR_NAMES = {1: "invalid argument", 2: "CUDA error", 3: "unsupported", 4: "wrong device"}


class NativeUnavailable(ImportError):
    """The compiled engine library is missing or could not be loaded."""


class NativeError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, fn: str, code: int, msg: str):
        super().__init__(f"{fn}: {ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


_lock = threading.Lock()
_lib = None


def load(path: Path | str | None = None):
    """Load (once) and return the ctypes library with every signature declared."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise NativeUnavailable(
                f"emsim_gb300 native library not found at {p}; build it with `python -m emsim_gb300.build`")
        try:
            lib = ctypes.CDLL(str(p))
        except OSError as e:  # pragma: no cover - depends on the host
            raise NativeUnavailable(f"cannot load {p}: {e}") from e
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if path is None:
            _lib = lib
        return lib


def call(name: str, *args) -> None:
    """Call a status-returning entry point and raise NativeError on failure."""
    lib = load()
    st = getattr(lib, name)(*args)
    if st != 0:
        raise NativeError(name, st, lib.emsim_gb300_last_error().decode(errors="replace"))


def last_error() -> str:
    return load().emsim_gb300_last_error().decode(errors="replace")


class DeviceWaitTimeout(RuntimeError):
    """A pipelined kernel's bounded wait for a tile copy gave up; the results of the work
    queued before this was noticed are invalid.  The device error word stays set until
    :func:`check_device_error` reads and clears it."""


def peek_device_error() -> int:
    """The current device's error word, read without synchronising or clearing it (kernels
    that have not finished yet are not reflected)."""
    code = ctypes.c_int(0)
    call("emsim_gb300_peek_device_error", ctypes.byref(code))
    return int(code.value)


def raise_on_device_error() -> None:
    """Raise :class:`DeviceWaitTimeout` when the current device's error word is set.  Call
    it after the host has waited for the work it wants to vouch for."""
    code = peek_device_error()
    if code != 0:
        raise DeviceWaitTimeout(f"device error word = {code}: a kernel's bounded wait for a tile copy timed out; "
                                f"results computed since the last emsim_gb300_check_device_error are invalid")


def check_device_error() -> int:
    """Synchronise and read (and clear) the device error word; 0 = no kernel gave up."""
    code = ctypes.c_int(0)
    call("emsim_gb300_check_device_error", ctypes.byref(code))
    return code.value
