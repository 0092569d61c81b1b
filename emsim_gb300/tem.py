"""Microscope parameters (emsim/tem.py:36-88)."""
from __future__ import annotations

from typing import Tuple, Union

from . import wave
from .physics import (aberration, electron_relativity_gamma, electron_wave_length_angstrom, mtf,
                      scherzer_condition)


class TEM:
    def __init__(self, electron_dose: float, beam_energy_kev: float, cs_mm: float, defocus: float, aperture: float):
        self.electron_dose = electron_dose
        self.beam_energy_kev = beam_energy_kev
        self.cs_mm = cs_mm
        self.defocus = defocus
        self.aperture = aperture

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
