"""emsim backend classes on the GB300 engine - the plugin boundary.

emsim resolves three classes from the current backend at every call
(emsim/config.py:31-41): ``OneSliceBuilder``, ``MultiSlicesBuilder`` and
``WavePropagator``.  This module provides them with the reference's constructor
arguments, method names, argument meaning and return shapes
(backend/slice_builder_base.py:8-163, backend/wave_propagator_base.py:10-44,
backend/*_cuda.py), computing through the C ABI of ``include/emsim_gb300.h``.

Arrays: inputs may be numpy arrays, torch tensors (any device) or objects exposing
``__cuda_array_interface__`` (cupy); outputs are torch CUDA tensors of class
:class:`DeviceArray`, which add the ``.get()`` host copy that emsim's simulator calls
on GPU results (simulator.py:51-53).  Work is queued on the current torch CUDA stream.

Extensions beyond the reference signatures (all optional): a leading batch axis on
waves and slices, ``Pipe``-style fused image formation in ``WavePropagator.image``.
"""
from __future__ import annotations

import ctypes
import logging
import math
import threading
from typing import Dict, List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import _native, elem, physics

logger = logging.getLogger(__name__)


class DeviceArray(torch.Tensor):
    """A torch CUDA tensor with ``get()`` returning a numpy copy (cupy's spelling)."""

    def get(self) -> np.ndarray:
        """Host copy; raises ``DeviceWaitTimeout`` when a kernel of the device gave up a
        bounded wait (its results would be invalid)."""
        out = self.detach().cpu().numpy()
        if self.is_cuda:
            with torch.cuda.device(self.device):
                _native.raise_on_device_error()
        return out


def _wrap(t: torch.Tensor) -> DeviceArray:
    return t.as_subclass(DeviceArray)


def _device() -> torch.device:
    if not torch.cuda.is_available():
        raise RuntimeError("emsim_gb300 needs a CUDA device")
    return torch.device("cuda", torch.cuda.current_device())


def _stream() -> ctypes.c_void_p:
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t: Optional[torch.Tensor]) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr() if t is not None else 0)


class Prepared:
    """Device work whose metadata already sits on the device and whose buffers are
    allocated: calling it makes only native calls on the current stream (no allocation,
    no host-to-device copy, no synchronisation), so it can be captured in a CUDA graph
    and replayed.  ``result`` is the tensor it writes; ``keep`` holds what the calls
    read (device metadata, workspaces, host scalars' arrays)."""

    __slots__ = ("_fn", "result", "_keep")

    def __init__(self, fn, result: torch.Tensor, keep=()):
        self._fn, self.result, self._keep = fn, result, keep

    def __call__(self) -> torch.Tensor:
        self._fn()
        return self.result


def as_device(x, dtype: torch.dtype) -> torch.Tensor:
    """Contiguous tensor of ``dtype`` on the current CUDA device (copy only if needed)."""
    dev = _device()
    if isinstance(x, torch.Tensor):
        t = x
    elif hasattr(x, "__cuda_array_interface__"):
        t = torch.as_tensor(x, device=dev)
    else:
        t = torch.from_numpy(np.ascontiguousarray(np.asarray(x)))
    if t.dtype != dtype:
        t = t.to(dtype)
    if t.device != dev:
        t = t.to(dev, non_blocking=False)
    return t.contiguous()


# ---------------------------------------------------------------------------------
# native plans (cached: the reference builds a new propagator and FFT plan per image,
# pipe.py:31-34; plans here depend only on geometry and are reused)
# ---------------------------------------------------------------------------------
class _Plan:
    def __init__(self, handle: ctypes.c_void_p, destroy: str):
        self.handle = handle
        self._destroy = destroy

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            if self.handle and _native._lib is not None:
                getattr(_native._lib, self._destroy)(self.handle)
        except Exception:
            pass


_plan_lock = threading.Lock()
_wave_plans: Dict[tuple, _Plan] = {}
_slice_plans: Dict[tuple, _Plan] = {}


def wave_plan(n1: int, n2: int, d1: float, d2: float, wave_length: float, gamma: float) -> _Plan:
    key = (torch.cuda.current_device(), n1, n2, float(d1), float(d2), float(wave_length), float(gamma))
    with _plan_lock:
        p = _wave_plans.get(key)
        if p is None:
            h = ctypes.c_void_p()
            _native.call("emsim_gb300_wave_plan_create", n1, n2, float(d1), float(d2), float(wave_length),
                         float(gamma), ctypes.byref(h))
            p = _wave_plans[key] = _Plan(h, "emsim_gb300_wave_plan_destroy")
        return p


def slice_plan(unique_elements: Sequence[int], n_slices: int, n1: int, n2: int, dz: float, d1: float, d2: float,
               bandlimit: bool = True) -> Tuple[_Plan, np.ndarray]:
    zs = tuple(sorted(int(z) for z in unique_elements))
    key = (torch.cuda.current_device(), zs, n_slices, n1, n2, float(dz), float(d1), float(d2), bool(bandlimit))
    sf = elem.scattering_factors_half(zs, n1, n2, d1, d2)
    with _plan_lock:
        p = _slice_plans.get(key)
        if p is None:
            h = ctypes.c_void_p()
            _native.call("emsim_gb300_slice_plan_create", sf.ctypes.data_as(ctypes.c_void_p), len(zs), n_slices, n1,
                         n2, float(dz), float(d1), float(d2), 1 if bandlimit else 0, ctypes.byref(h))
            p = _slice_plans[key] = _Plan(h, "emsim_gb300_slice_plan_destroy")
        return p, sf


# ---------------------------------------------------------------------------------
# slice builders
# ---------------------------------------------------------------------------------
def _bin(plan: _Plan, fn: str, coords, counts, out_shape) -> DeviceArray:
    dev = _device()
    c = as_device(coords, torch.float32).reshape(-1, 3)
    cnt = as_device(np.asarray(counts, dtype=np.int64).astype(np.uint32).view(np.int32), torch.int32) \
        if not isinstance(counts, torch.Tensor) else as_device(counts, torch.int32)
    if cnt.dim() != 1 or cnt.shape[0] != out_shape[0]:
        raise ValueError(f"unique_elements_count must have {out_shape[0]} entries, got {tuple(cnt.shape)}")
    out = torch.empty(out_shape, dtype=torch.float32, device=dev)
    _native.call(fn, plan.handle, _ptr(c), int(c.shape[0]), _ptr(cnt), _ptr(out), _stream())
    return _wrap(out)


def _make(plan: _Plan, hist, n_slices: int, n1: int, n2: int) -> torch.Tensor:
    dev = _device()
    h = as_device(hist, torch.float32)
    out = torch.empty((n_slices, n1, n2), dtype=torch.float32, device=dev)
    nbytes = int(_native.load().emsim_gb300_make_slices_workspace_size(plan.handle))
    work = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=dev)
    _native.call("emsim_gb300_make_slices", plan.handle, _ptr(h), _ptr(out), _ptr(work), nbytes, _stream())
    return out


class OneSliceBuilder:
    """One projected-potential slice (slice_builder_base.py:8-73, slice_builder_cuda.py:24-44)."""

    def __init__(self, unique_elements: List[int], n1: int, n2: int, d1: float, d2: float):
        self.n1, self.n2 = n1, n2
        self.d1, self.d2 = d1, d2
        self.unique_elements = unique_elements
        self._plan, self.scattering_factors = slice_plan(unique_elements, 1, n1, n2, 1.0, d1, d2, True)

    def bin_atoms_one_slice(self, atom_coordinates_sorted_by_elems, unique_elements_count):
        """(nE, n1, n2) float32 histogram of columns (x, y) = 1, 2."""
        return _bin(self._plan, "emsim_gb300_bin_atoms_one_slice", atom_coordinates_sorted_by_elems,
                    unique_elements_count, (len(self.unique_elements), self.n1, self.n2))

    def make_one_slice(self, atom_histograms_one_slice, symmetric_bandlimit: bool = True):
        """(n1, n2) float32 band-limited projected potential clipped at 1e-13."""
        plan = self._plan if symmetric_bandlimit else slice_plan(
            self.unique_elements, 1, self.n1, self.n2, 1.0, self.d1, self.d2, False)[0]
        return _wrap(_make(plan, atom_histograms_one_slice, 1, self.n1, self.n2)[0])


class MultiSlicesBuilder:
    """Stack of slices (slice_builder_base.py:76-163, slice_builder_cuda.py:47-85)."""

    def __init__(self, unique_elements: List[int], n_slices: int, n1: int, n2: int, dz: float, d1: float,
                 d2: float):
        self.n_slice = n_slices
        self.n1, self.n2 = n1, n2
        self.dz = dz
        self.d1, self.d2 = d1, d2
        self.unique_elements = unique_elements
        self._plan, self.scattering_factors = slice_plan(unique_elements, n_slices, n1, n2, dz, d1, d2, True)

    def bin_atoms_multi_slices(self, atom_coordinates_sorted_by_elems, unique_elements_count):
        """(nE, n_slices, n1, n2) float32 histogram of columns (z, x, y)."""
        return _bin(self._plan, "emsim_gb300_bin_atoms_multi_slices", atom_coordinates_sorted_by_elems,
                    unique_elements_count, (len(self.unique_elements), self.n_slice, self.n1, self.n2))

    def add_water(self, atom_histograms, seed: Optional[int] = None, stream_id: int = 0):
        """Voxel water (slice_builder_base.py:134-147): in voxels empty for every element,
        add Poisson(0.031 d1 d2 dz) oxygens and Poisson(2x that) hydrogens.  Z = 1 and 8
        must be among the unique elements.  The draws are counter-based (Philox4x32-10,
        ``emsim_gb300_add_water``): ``seed`` reproduces them; without one a seed is drawn
        from numpy's global generator, the generator the reference draws from."""
        h = as_device(atom_histograms, torch.float32)
        zs = list(self.unique_elements)
        if 1 not in zs or 8 not in zs:
            raise ValueError("add_water needs Z = 1 and Z = 8 among the unique elements")
        if seed is None:
            seed = int(np.random.randint(0, 2 ** 62, dtype=np.int64))
        _native.call("emsim_gb300_add_water", self._plan.handle, _ptr(h), zs.index(1), zs.index(8),
                     float(physics.water_num_dens), int(seed) & (2 ** 64 - 1), int(stream_id) & 0xFFFFFFFF, _stream())
        return _wrap(h)

    def make_multi_slices(self, atom_histograms, symmetric_bandlimit: bool = True):
        """(n_slices, n1, n2) float32 band-limited slices clipped at 1e-13."""
        plan = self._plan if symmetric_bandlimit else slice_plan(
            self.unique_elements, self.n_slice, self.n1, self.n2, self.dz, self.d1, self.d2, False)[0]
        return _wrap(_make(plan, atom_histograms, self.n_slice, self.n1, self.n2))

    @property
    def atoms_path(self) -> bool:
        """True when slices can be built straight from atoms (power-of-two sides 8..4096)."""
        return all(n >= 8 and n <= 4096 and n & (n - 1) == 0 for n in (self.n1, self.n2))

    def build_from_atoms(self, atom_coordinates_sorted_by_elems, unique_elements_count,
                         symmetric_bandlimit: bool = True):
        """make_multi_slices(bin_atoms_multi_slices(...)) without the dense histogram:
        (n_slices, n1, n2) float32."""
        return build_slices_batch(self, [(atom_coordinates_sorted_by_elems, unique_elements_count)],
                                  symmetric_bandlimit)[0]


def _element_slots(builder: MultiSlicesBuilder) -> np.ndarray:
    eoz = np.full(128, -1, dtype=np.int32)
    for k, zz in enumerate(sorted(int(v) for v in builder.unique_elements)):
        if 0 <= zz < 128:
            eoz[zz] = k
    return eoz


def prepare_build_slices_from_device_atoms(builder: MultiSlicesBuilder, xyz: torch.Tensor, z: torch.Tensor,
                                           offsets: torch.Tensor, shift: torch.Tensor, mol_index: Sequence[int],
                                           n_mol: int, symmetric_bandlimit: bool = True,
                                           slot_slices: Optional[Sequence[int]] = None) -> Prepared:
    """:func:`build_slices_from_device_atoms` with its metadata uploaded and its output and
    workspace allocated; calling the result runs the build."""
    plan = builder._plan if symmetric_bandlimit else slice_plan(
        builder.unique_elements, builder.n_slice, builder.n1, builder.n2, builder.dz, builder.d1, builder.d2,
        False)[0]
    dev = _device()
    slot = np.full(n_mol, -1, dtype=np.int32)
    slot[list(mol_index)] = np.arange(len(mol_index), dtype=np.int32)
    nb = len(mol_index)
    parts = [slot, _element_slots(builder)]
    if slot_slices is not None:
        ss = np.asarray(slot_slices, dtype=np.int32).reshape(-1)
        if ss.shape[0] != nb or ss.min(initial=1) < 1 or ss.max(initial=1) > builder.n_slice:
            raise ValueError(f"slot_slices must hold {nb} counts in [1, {builder.n_slice}]")
        parts.append(ss)
    meta = torch.from_numpy(np.concatenate(parts)).to(dev, non_blocking=True)
    n_atoms = int(xyz.shape[0])
    out = torch.empty((nb, builder.n_slice, builder.n1, builder.n2), dtype=torch.float32, device=dev)
    nbytes = int(_native.load().emsim_gb300_build_slices_workspace_size(plan.handle, n_atoms, nb))
    ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=dev)
    eoz_ptr = ctypes.c_void_p(meta.data_ptr() + 4 * n_mol)

    def run():
        if slot_slices is None:
            _native.call("emsim_gb300_build_slices_z", plan.handle, _ptr(xyz), _ptr(z), n_atoms, _ptr(offsets),
                         n_mol, _ptr(shift), _ptr(meta), eoz_ptr, nb, _ptr(out), _ptr(ws), nbytes, _stream())
        else:
            _native.call("emsim_gb300_build_slices_ragged", plan.handle, _ptr(xyz), _ptr(z), n_atoms, _ptr(offsets),
                         n_mol, _ptr(shift), _ptr(meta), eoz_ptr,
                         ctypes.c_void_p(meta.data_ptr() + 4 * (n_mol + 128)), nb, _ptr(out), _ptr(ws), nbytes,
                         _stream())

    return Prepared(run, out, (plan, meta, ws, xyz, z, offsets, shift))


def build_slices_from_device_atoms(builder: MultiSlicesBuilder, xyz: torch.Tensor, z: torch.Tensor,
                                   offsets: torch.Tensor, shift: torch.Tensor, mol_index: Sequence[int], n_mol: int,
                                   symmetric_bandlimit: bool = True,
                                   slot_slices: Optional[Sequence[int]] = None) -> DeviceArray:
    """Slices of molecules ``mol_index`` of a device-resident batch: ``xyz`` (n_atoms, 3)
    float32, ``z`` (n_atoms) int32, ``offsets`` (n_mol + 1) uint32 atom offsets, ``shift``
    (n_mol, 3) float32 per-molecule translation (centralisation).  Returns
    (len(mol_index), n_slices, n1, n2) float32.  ``slot_slices``: each molecule's own slice
    count (<= builder.n_slice; ragged batch): molecule k is binned on the slice axis of
    its own count and fills slices [0, slot_slices[k]) of its stack."""
    return _wrap(prepare_build_slices_from_device_atoms(builder, xyz, z, offsets, shift, mol_index, n_mol,
                                                        symmetric_bandlimit, slot_slices)())


def prepare_image_from_device_atoms(builder: MultiSlicesBuilder, wp: "WavePropagator", xyz: torch.Tensor,
                                    z: torch.Tensor, offsets: torch.Tensor, shift: torch.Tensor,
                                    mol_index: Sequence[int], n_mol: int, electron_dose: float, cs_mm: float, defocus,
                                    aperture: float, chunk_pairs: int = 0) -> Prepared:
    """:func:`image_from_device_atoms` with its metadata uploaded and its image and
    workspace allocated; calling the result forms the images."""
    plan = builder._plan
    dev = _device()
    slot = np.full(n_mol, -1, dtype=np.int32)
    slot[list(mol_index)] = np.arange(len(mol_index), dtype=np.int32)
    nb = len(mol_index)
    meta = torch.from_numpy(np.concatenate([slot, _element_slots(builder)])).to(dev, non_blocking=True)
    n_atoms = int(xyz.shape[0])
    lib = _native.load()
    nbytes = int(lib.emsim_gb300_image_from_atoms_workspace_size(plan.handle, n_atoms, nb, int(chunk_pairs)))
    ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=dev)
    img = torch.empty((nb, builder.n1, builder.n2), dtype=torch.float32, device=dev)
    dfs = np.ascontiguousarray(np.atleast_1d(np.asarray(defocus, dtype=np.float64)))

    def run():
        _native.call("emsim_gb300_image_from_atoms_z", plan.handle, wp._plan.handle, _ptr(xyz), _ptr(z), n_atoms,
                     _ptr(offsets), n_mol, _ptr(shift), _ptr(meta), ctypes.c_void_p(meta.data_ptr() + 4 * n_mol), nb,
                     float(electron_dose), float(cs_mm), dfs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                     len(dfs), float(aperture), _ptr(img), int(chunk_pairs), _ptr(ws), nbytes, _stream())

    return Prepared(run, img, (plan, wp, meta, ws, dfs, xyz, z, offsets, shift))


def image_from_device_atoms(builder: MultiSlicesBuilder, wp: "WavePropagator", xyz: torch.Tensor, z: torch.Tensor,
                            offsets: torch.Tensor, shift: torch.Tensor, mol_index: Sequence[int], n_mol: int,
                            electron_dose: float, cs_mm: float, defocus, aperture: float,
                            chunk_pairs: int = 0) -> DeviceArray:
    """Images of molecules ``mol_index`` of a device-resident batch (arguments as for
    :func:`build_slices_from_device_atoms`) with the slices built ``chunk_pairs`` slice
    pairs at a time (``emsim_gb300_image_from_atoms_z``): the slice stack is never held
    whole, and the images are bitwise those of build_slices_from_device_atoms followed
    by ``WavePropagator.image``.  Returns (len(mol_index), n1, n2) float32."""
    return _wrap(prepare_image_from_device_atoms(builder, wp, xyz, z, offsets, shift, mol_index, n_mol,
                                                 electron_dose, cs_mm, defocus, aperture, chunk_pairs)())


def build_slices_batch(builder: MultiSlicesBuilder, mols, symmetric_bandlimit: bool = True) -> DeviceArray:
    """Slices of several molecules in one engine call.  ``mols``: sequence of
    (coordinates sorted by element (N_b, 3), per-element counts in the builder's
    element order).  Returns (B, n_slices, n1, n2) float32."""
    if not builder.atoms_path:
        return _wrap(torch.stack([builder.make_multi_slices(builder.bin_atoms_multi_slices(c, n), symmetric_bandlimit)
                                  for c, n in mols]))
    plan = builder._plan if symmetric_bandlimit else slice_plan(
        builder.unique_elements, builder.n_slice, builder.n1, builder.n2, builder.dz, builder.d1, builder.d2,
        False)[0]
    dev = _device()
    n_e = len(builder.unique_elements)
    counts = np.zeros((len(mols), n_e), dtype=np.uint32)
    parts = []
    for i, (c, n) in enumerate(mols):
        n = np.asarray(n).reshape(-1)
        if n.shape[0] != n_e:
            raise ValueError(f"unique_elements_count must have {n_e} entries, got {n.shape[0]}")
        counts[i] = n
        parts.append(np.asarray(c, dtype=np.float32).reshape(-1, 3) if not isinstance(c, torch.Tensor)
                     else c.detach().to("cpu", torch.float32).numpy().reshape(-1, 3))
    xyz = np.ascontiguousarray(np.concatenate(parts) if parts else np.zeros((0, 3), np.float32))
    c_dev = as_device(xyz, torch.float32)
    n_dev = as_device(counts.view(np.int32), torch.int32)
    n_atoms = int(xyz.shape[0])
    out = torch.empty((len(mols), builder.n_slice, builder.n1, builder.n2), dtype=torch.float32, device=dev)
    lib = _native.load()
    nbytes = int(lib.emsim_gb300_build_slices_workspace_size(plan.handle, n_atoms, len(mols)))
    ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=dev)
    _native.call("emsim_gb300_build_slices", plan.handle, _ptr(c_dev), n_atoms, _ptr(n_dev), len(mols), _ptr(out),
                 _ptr(ws), nbytes, _stream())
    return _wrap(out)


# ---------------------------------------------------------------------------------
# wave propagator
# ---------------------------------------------------------------------------------
class WavePropagator:
    """Raw wave propagator (wave_propagator_base.py:10-44, wave_propagator_cuda.py:21-60).

    All methods are out-of-place and return complex64 (n1, n2) (or (B, n1, n2) for a
    batch of B waves) DeviceArrays.  FFT semantics follow the reference's native
    backends: true fftfreq grid, 2/3 band-limit in every propagation, aperture
    f^2 <= (alpha/lambda)^2.
    """

    def __init__(self, n1: int, n2: int, d1: float, d2: float, beam_energy_kev: float):
        self.wave_shape = (n1, n2)
        self.d1, self.d2 = d1, d2
        self.wave_length = physics.electron_wave_length_angstrom(beam_energy_kev)
        self.relativity_gamma = physics.electron_relativity_gamma(beam_energy_kev)
        self._plan = wave_plan(n1, n2, d1, d2, self.wave_length, self.relativity_gamma)

    # -- helpers ----------------------------------------------------------------
    def _wave(self, wave) -> Tuple[torch.Tensor, int]:
        w = as_device(wave, torch.complex64)
        n1, n2 = self.wave_shape
        if w.dim() == 2 and tuple(w.shape) == (n1, n2):
            return w, 1
        if w.dim() == 3 and tuple(w.shape[1:]) == (n1, n2):
            return w, int(w.shape[0])
        raise ValueError(f"wave must be ({n1}, {n2}) or (B, {n1}, {n2}), got {tuple(w.shape)}")

    def _slice(self, aslice, nb: int) -> Tuple[torch.Tensor, int]:
        s = as_device(aslice, torch.float32)
        n1, n2 = self.wave_shape
        if tuple(s.shape) == (n1, n2):
            return s, 0
        if s.dim() == 3 and tuple(s.shape) == (nb, n1, n2):
            return s, n1 * n2
        raise ValueError(f"slice must be ({n1}, {n2}) or ({nb}, {n1}, {n2}), got {tuple(s.shape)}")

    def _stack(self, slices, nb: int) -> Tuple[torch.Tensor, int, int]:
        s = as_device(slices, torch.float32)
        n1, n2 = self.wave_shape
        if s.dim() == 3 and tuple(s.shape[1:]) == (n1, n2):
            return s, int(s.shape[0]), 0
        if s.dim() == 4 and s.shape[0] == nb and tuple(s.shape[2:]) == (n1, n2):
            return s, int(s.shape[1]), int(s.shape[1]) * n1 * n2
        raise ValueError(f"slices must be (n_slices, {n1}, {n2}) or ({nb}, n_slices, {n1}, {n2})")

    # -- the reference API ------------------------------------------------------
    def init_wave(self, electron_dose: float):
        out = torch.empty(self.wave_shape, dtype=torch.complex64, device=_device())
        _native.call("emsim_gb300_init_wave", self._plan.handle, float(electron_dose), _ptr(out), 1, _stream())
        return _wrap(out)

    def slice_transmit(self, wave, aslice):
        w, nb = self._wave(wave)
        s, sstride = self._slice(aslice, nb)
        out = torch.empty_like(w)
        _native.call("emsim_gb300_slice_transmit", self._plan.handle, _ptr(w), _ptr(s), sstride, _ptr(out), nb,
                     _stream())
        return _wrap(out)

    def space_propagate(self, wave, dz: float):
        w, nb = self._wave(wave)
        out = torch.empty_like(w)
        _native.call("emsim_gb300_space_propagate", self._plan.handle, _ptr(w), float(dz), _ptr(out), nb, _stream())
        return _wrap(out)

    def singleslice_propagate(self, wave, aslice, dz: float):
        w, nb = self._wave(wave)
        s, sstride = self._slice(aslice, nb)
        out = torch.empty_like(w)
        _native.call("emsim_gb300_singleslice_propagate", self._plan.handle, _ptr(w), _ptr(s), sstride, float(dz),
                     _ptr(out), nb, _stream())
        return _wrap(out)

    def multislice_propagate(self, wave, slices, dz: float):
        w, nb = self._wave(wave)
        s, ns, sstride = self._stack(slices, nb)
        out = torch.empty_like(w)
        _native.call("emsim_gb300_multislice_propagate", self._plan.handle, _ptr(w), _ptr(s), ns, sstride, float(dz),
                     _ptr(out), nb, _stream())
        return _wrap(out)

    def lens_propagate(self, wave, cs_mm: float, defocus: float, aperture: float):
        w, nb = self._wave(wave)
        out = torch.empty_like(w)
        _native.call("emsim_gb300_lens_propagate", self._plan.handle, _ptr(w), float(cs_mm), float(defocus),
                     float(aperture), _ptr(out), nb, _stream())
        return _wrap(out)

    # -- partial coherence (extension) ---------------------------------------------
    def lens_intensity_incoherent(self, exit_wave, cs_mm: float, defocus_values, weights, aperture: float,
                                  illumination_angle: float = 0.0) -> DeviceArray:
        """sum_k weights[k] * |lens(exit_wave, defocus_values[k])|^2, each lens transfer damped
        by the quasi-coherent envelope of an illumination semi-angle (rad; 0 = coherent)
        (``emsim_gb300_lens_intensity_incoherent``).  (n1, n2) or (B, n1, n2) float32."""
        w, nb = self._wave(exit_wave)
        d = np.ascontiguousarray(np.atleast_1d(np.asarray(defocus_values, dtype=np.float64)))
        wt = np.ascontiguousarray(np.atleast_1d(np.asarray(weights, dtype=np.float64)))
        if d.ndim != 1 or d.shape != wt.shape or d.size < 1:
            raise ValueError("defocus_values and weights must be equal-length 1-D sequences")
        n1, n2 = self.wave_shape
        out = torch.empty((nb, n1, n2), dtype=torch.float32, device=_device())
        lib = _native.load()
        nbytes = int(lib.emsim_gb300_lens_incoherent_workspace_size(self._plan.handle, nb))
        work = torch.empty(nbytes, dtype=torch.uint8, device=_device())
        dp = ctypes.POINTER(ctypes.c_double)
        _native.call("emsim_gb300_lens_intensity_incoherent", self._plan.handle, _ptr(w), nb, float(cs_mm),
                     d.ctypes.data_as(dp), wt.ctypes.data_as(dp), int(d.size), float(illumination_angle),
                     float(aperture), _ptr(out), _ptr(work), nbytes, _stream())
        return _wrap(out[0] if w.dim() == 2 else out)

    def image_partially_coherent(self, slices, dz: float, electron_dose: float, cs_mm: float, defocus: float,
                                 aperture: float, focal_spread: float = 0.0, illumination_angle: float = 0.0,
                                 n_focal: int = 7, n_batch: Optional[int] = None) -> DeviceArray:
        """Plane wave -> multislice -> partially coherent lens -> intensity: the focal spread
        (standard deviation of the defocus, A) as an incoherent sum over n_focal
        Gauss-Hermite defocus values, the illumination semi-angle (rad) as the
        quasi-coherent spatial envelope.  ``slices``: (n_slices, n1, n2) shared by n_batch
        images (default 1) or (B, n_slices, n1, n2)."""
        s = as_device(slices, torch.float32)
        nb = int(s.shape[0]) if s.dim() == 4 else (n_batch or 1)
        n1, n2 = self.wave_shape
        psi = torch.empty((nb, n1, n2), dtype=torch.complex64, device=_device())
        _native.call("emsim_gb300_init_wave", self._plan.handle, float(electron_dose), _ptr(psi), nb, _stream())
        ew = self.multislice_propagate(psi, s, dz)
        dfs, wts = focal_spread_quadrature(defocus, focal_spread, n_focal)
        img = self.lens_intensity_incoherent(ew, cs_mm, dfs, wts, aperture, illumination_angle)
        return _wrap(img.reshape(n1, n2)) if s.dim() == 3 and n_batch is None else img

    # -- fused image formation (extension) --------------------------------------
    def image(self, slices, dz: float, electron_dose: float, cs_mm: float, defocus, aperture: float,
              n_batch: Optional[int] = None, return_exit_wave: bool = False):
        """init_wave -> multislice -> lens -> |psi|^2 in one call (pipe.py:46-55, 79-84).

        ``slices``: (n_slices, n1, n2) shared or (B, n_slices, n1, n2); ``defocus``: a
        number or a sequence (image b uses defocus[b % len]).  Returns (n1, n2) or
        (B, n1, n2) float32 intensities (and the exit waves when requested)."""
        s = as_device(slices, torch.float32)
        prep = self.prepare_image(s, dz, electron_dose, cs_mm, defocus, aperture, n_batch, return_exit_wave)
        img = prep()
        squeeze = s.dim() == 3 and n_batch is None and not np.ndim(defocus)
        out = _wrap(img[0] if squeeze else img)
        if return_exit_wave:
            ew = prep._keep[-1]
            return out, _wrap(ew[0] if squeeze else ew)
        return out

    def prepare_image(self, slices: torch.Tensor, dz: float, electron_dose: float, cs_mm: float, defocus,
                      aperture: float, n_batch: Optional[int] = None, return_exit_wave: bool = False) -> Prepared:
        """:meth:`image` on device slices with its buffers allocated; calling the result
        forms the (B, n1, n2) images (the exit waves, when requested, in ``_keep[-1]``)."""
        n1, n2 = self.wave_shape
        s = slices
        if s.dim() == 4:
            nb, ns, sstride = int(s.shape[0]), int(s.shape[1]), int(s.shape[1]) * n1 * n2
        else:
            ns, sstride = int(s.shape[0]), 0
            nb = n_batch or (len(defocus) if np.ndim(defocus) else 1)
        dfs = np.ascontiguousarray(np.atleast_1d(np.asarray(defocus, dtype=np.float64)))
        dev = _device()
        img = torch.empty((nb, n1, n2), dtype=torch.float32, device=dev)
        work = torch.empty((nb, n1, n2), dtype=torch.complex64, device=dev)
        ew = torch.empty_like(work) if return_exit_wave else None

        def run():
            _native.call("emsim_gb300_multislice_image", self._plan.handle, _ptr(s), ns, sstride, float(dz),
                         float(electron_dose), float(cs_mm), dfs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                         len(dfs), float(aperture), _ptr(img), _ptr(work), _ptr(ew), nb, _stream())

        return Prepared(run, img, (self._plan, s, dfs, work, ew))


def focal_spread_quadrature(defocus: float, focal_spread: float, n: int = 7) -> Tuple[np.ndarray, np.ndarray]:
    """Defocus values and weights of an n-point Gauss-Hermite rule for a Gaussian defocus
    distribution (mean ``defocus``, standard deviation ``focal_spread``, A); the weights
    sum to one.  focal_spread = 0 gives the single coherent defocus."""
    if focal_spread < 0 or n < 1:
        raise ValueError("focal_spread must be >= 0 and n >= 1")
    if focal_spread == 0:
        return np.array([float(defocus)]), np.array([1.0])
    x, w = np.polynomial.hermite.hermgauss(int(n))
    return float(defocus) + math.sqrt(2.0) * float(focal_spread) * x, w / math.sqrt(math.pi)


def prepare_image_ragged(wp: "WavePropagator", stacks: torch.Tensor, n_slices: Sequence[int], dz: float,
                         electron_dose: float, cs_mm: float, defocus, aperture: float) -> Prepared:
    """:func:`image_ragged` for device stacks already ordered longest first, with its
    buffers allocated; calling the result forms the images (in the stacks' order)."""
    s = stacks
    nb, smax, n1, n2 = (int(x) for x in s.shape)
    ns = np.ascontiguousarray(np.asarray(n_slices, dtype=np.int32).reshape(-1))
    if ns.shape[0] != nb or ns.min(initial=1) < 1 or ns.max(initial=1) > smax:
        raise ValueError(f"n_slices must hold {nb} counts in [1, {smax}]")
    if np.any(np.diff(ns) > 0):
        raise ValueError("prepare_image_ragged wants the stacks ordered by slice count, longest first")
    dfs = np.ascontiguousarray(np.atleast_1d(np.asarray(defocus, dtype=np.float64)))
    img = torch.empty((nb, n1, n2), dtype=torch.float32, device=s.device)
    work = torch.empty((nb, n1, n2), dtype=torch.complex64, device=s.device)

    def run():
        _native.call("emsim_gb300_multislice_image_ragged", wp._plan.handle, _ptr(s), smax * n1 * n2,
                     ns.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), float(dz), float(electron_dose),
                     float(cs_mm), dfs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(dfs), float(aperture),
                     _ptr(img), _ptr(work), nb, _stream())

    return Prepared(run, img, (wp._plan, s, ns, dfs, work))


def image_ragged(wp: "WavePropagator", stacks, n_slices: Sequence[int], dz: float, electron_dose: float,
                 cs_mm: float, defocus, aperture: float) -> DeviceArray:
    """Images of a ragged batch: ``stacks`` (B, S_max, n1, n2) float32 where image b uses
    its first n_slices[b] slices.  Images are propagated longest first, each step only
    over the images that still have a slice (``emsim_gb300_multislice_image_ragged``);
    results come back in input order, (B, n1, n2) float32."""
    s = as_device(stacks, torch.float32)
    nb, smax = int(s.shape[0]), int(s.shape[1])
    ns = np.asarray(n_slices, dtype=np.int32).reshape(-1)
    if ns.shape[0] != nb or ns.min(initial=1) < 1 or ns.max(initial=1) > smax:
        raise ValueError(f"n_slices must hold {nb} counts in [1, {smax}]")
    dfs = np.atleast_1d(np.asarray(defocus, dtype=np.float64))
    order = np.argsort(-ns, kind="stable")
    dev = s.device
    if np.any(order != np.arange(nb)):
        s = s[torch.as_tensor(order, device=dev)].contiguous()
        dfs = np.ascontiguousarray(np.resize(dfs, nb)[order]) if dfs.size > 1 else dfs
    img = prepare_image_ragged(wp, s, ns[order], dz, electron_dose, cs_mm, dfs, aperture)()
    if np.any(order != np.arange(nb)):
        inv = np.empty(nb, dtype=np.int64)
        inv[order] = np.arange(nb)
        img = img[torch.as_tensor(inv, device=dev)]
    return _wrap(img)


PRECISIONS = {"fp32": 0, "bf16x3": 1}


def set_precision(mode: str) -> None:
    """Precision of the wave passes, process-wide: "fp32" (plain FP32 Stockham FFTs, the
    default) or "bf16x3" (256-point rows and columns of the multislice step on the tensor
    cores as split-BF16 DFT GEMMs with fp32 accumulation; other sizes stay FP32)."""
    if mode not in PRECISIONS:
        raise ValueError(f"precision must be one of {sorted(PRECISIONS)}")
    _native.call("emsim_gb300_set_precision", PRECISIONS[mode])


def get_precision() -> str:
    v = int(_native.load().emsim_gb300_get_precision())
    return {k: m for m, k in PRECISIONS.items()}[v]


def intensity(wave) -> DeviceArray:
    """|psi|^2 of a complex64 array through the engine."""
    w = as_device(wave, torch.complex64)
    out = torch.empty(w.shape, dtype=torch.float32, device=w.device)
    _native.call("emsim_gb300_intensity", _ptr(w), _ptr(out), w.numel(), _stream())
    return _wrap(out)
