"""Microscope parameters and specimen container (emsim/tem.py:9-108)."""
from __future__ import annotations

from typing import Tuple, Union

import torch

from . import _native, wave
from .backend import _ptr, _stream, _wrap, as_device
from .physics import (aberration, electron_relativity_gamma, electron_wave_length_angstrom, mtf,
                      scherzer_condition)


class Specimen:
    """Slices (n_slices, n1, n2) with their pixel size and thickness (emsim/tem.py:9-33)."""

    def __init__(self, slices, pixel_size, dz):
        self.slices = slices
        self.pixel_size = pixel_size
        self.dz = dz

    @property
    def lateral_size(self):
        return tuple(self.slices.shape[1:])

    @property
    def num_slices(self):
        return self.slices.shape[0]

    def __iter__(self):
        self._s = 0
        return self

    def __next__(self):
        if self._s < self.num_slices:
            slc = self.slices[self._s, ...]
            self._s += 1
            return slc
        raise StopIteration


def band_limit_specimen(specimen: Specimen) -> Specimen:
    """Low-pass every slice with the disc of radius 2/3 * min(n1, n2)//2 on the centred
    frequency grid and keep the real part (emsim/tem.py:102-108), on the device
    (``emsim_gb300_band_limit_slices``).  The reference transforms axes (0, 1) of its
    stack, which agrees with its own (n_slices, n1, n2) layout only for cubic stacks; here
    each slice is filtered on its lateral axes."""
    s = as_device(specimen.slices, torch.float32)
    if s.dim() == 2:
        s = s[None]
    ns, n1, n2 = (int(x) for x in s.shape)
    out = torch.empty_like(s)
    nbytes = int(_native.load().emsim_gb300_band_limit_workspace_size(ns, n1, n2))
    ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=s.device)
    _native.call("emsim_gb300_band_limit_slices", _ptr(s), ns, n1, n2, _ptr(out), _ptr(ws), nbytes, _stream())
    return Specimen(_wrap(out), specimen.pixel_size, specimen.dz)


class TEM:
    """Microscope parameters (tem.py).  Extension: ``focal_spread`` (standard deviation of
    the defocus, A) and ``illumination_angle`` (semi-angle, rad) make images partially
    coherent (focal spread as an incoherent sum over ``n_focal`` Gauss-Hermite defocus
    values, illumination as the quasi-coherent spatial envelope); both 0 by default, which
    is the reference's coherent imaging."""

    def __init__(self, electron_dose: float, beam_energy_kev: float, cs_mm: float, defocus: float, aperture: float,
                 focal_spread: float = 0.0, illumination_angle: float = 0.0, n_focal: int = 7):
        self.electron_dose = electron_dose
        self.beam_energy_kev = beam_energy_kev
        self.cs_mm = cs_mm
        self.defocus = defocus
        self.aperture = aperture
        self.focal_spread = focal_spread
        self.illumination_angle = illumination_angle
        self.n_focal = n_focal

    @property
    def partially_coherent(self) -> bool:
        return self.focal_spread > 0 or self.illumination_angle > 0

    @property
    def relativity_gamma(self):
        return electron_relativity_gamma(self.beam_energy_kev)

    @property
    def wave_length(self):
        return electron_wave_length_angstrom(self.beam_energy_kev)

    def get_mtf_function(self):
        return mtf(self.wave_length, self.cs_mm, self.defocus)

    def get_ctf_function(self):
        return lambda k: -mtf(self.wave_length, self.cs_mm, self.defocus)(k).imag

    def get_aberration_function(self):
        return aberration(self.wave_length, self.cs_mm, self.defocus)

    def get_wave_propagator(self, wave_shape: Union[int, Tuple[int, int]],
                            pixel_size: Union[float, Tuple[float, float]]):
        return wave.WavePropagator(wave_shape, pixel_size, self.beam_energy_kev, self.electron_dose, self.cs_mm,
                                   self.defocus, self.aperture)

    def set_scherzer_condition(self):
        self.defocus, self.aperture = scherzer_condition(self.wave_length, self.cs_mm)

    def __repr__(self):
        return (f"{{TEM | beam_energy = {self.beam_energy_kev:.2f}keV, cs = {self.cs_mm:.2f}mm, "
                f"defocus = {0.1 * self.defocus:.2f}nm, aperture = {self.aperture:.2f} rad}}")
