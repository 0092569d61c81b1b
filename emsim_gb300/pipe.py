"""Imaging pipeline (emsim/pipe.py:9-91) on the GB300 backend.

``Pipe.run`` keeps the reference's semantics - centralize, build the slices with
lateral size ``roi`` and thickness ``slice_thickness`` (optionally with voxel water),
plane wave, multislice, objective lens, |psi|^2 - and forms the image in one fused
engine call after the slices exist.  ``run_batch`` forms many images, one engine call
per group of equal (n_slices, roi).
"""
from __future__ import annotations

from collections import defaultdict
from typing import List, Optional, Sequence, Tuple, Union

import numpy as np
import torch

from . import atoms as atm
from . import backend, pot, tem, wave


class Pipe:
    def __init__(self, microscope: tem.TEM, resolution: float, slice_thickness: float,
                 roi: Optional[Union[int, Tuple[int, int]]] = None, n_slices: Optional[int] = None,
                 add_water: bool = True, upto_exit_wave: bool = False):
        self._resolution = resolution
        self._pixel_size = 0.5 * resolution
        self.microscope = microscope
        self.slice_thickness = slice_thickness
        self.add_water = add_water
        self.upto_exit_wave = upto_exit_wave
        self.roi = (roi, roi) if type(roi) is int else roi
        # stored but, as in the reference (pipe.py:48-52), not used to size the slices
        self.n_slices = n_slices

    @property
    def resolution(self):
        return self._resolution

    @resolution.setter
    def resolution(self, res):
        self._pixel_size = 0.5 * res
        self._resolution = res

    def _propagator(self, shape):
        return wave.get_raw_wave_propagator(tuple(shape), self._pixel_size, self.microscope.beam_energy_kev)

    @property
    def wave_propagator(self):
        return self._propagator(self.roi)

    def build_slices(self, mol: atm.AtomList):
        mol = atm.centralize(mol)
        return pot.build_multi_slices(mol, dz=self.slice_thickness, pixel_size=self._pixel_size,
                                      lateral_size=self.roi, add_water=self.add_water)

    def get_exit_wave(self, mol):
        slices = self.build_slices(mol)
        wp = self._propagator(slices.shape[-2:])
        return wp.multislice_propagate(wp.init_wave(self.microscope.electron_dose), slices, self.slice_thickness)

    def get_exit_wave_wpo(self, mol):
        mol = atm.centralize(mol)
        aslice = pot.build_one_slice(mol, pixel_size=self._pixel_size, lateral_size=self.roi)
        wp = self._propagator(aslice.shape[-2:])
        return wp.singleslice_propagate(wp.init_wave(self.microscope.electron_dose), aslice, dz=0)

    def lens_propagate(self, exit_wave):
        m = self.microscope
        wp = self._propagator(exit_wave.shape[-2:])
        return wp.lens_propagate(exit_wave, m.cs_mm, m.defocus, m.aperture)

    def run_wpo(self, mol):
        iw = self.lens_propagate(self.get_exit_wave_wpo(mol))
        return iw.real ** 2 + iw.imag ** 2

    def run(self, mol):
        """Image of one molecule, (n1, n2) float32 on the device."""
        slices = self.build_slices(mol)
        m = self.microscope
        wp = self._propagator(slices.shape[-2:])
        return wp.image(slices, self.slice_thickness, m.electron_dose, m.cs_mm, m.defocus, m.aperture)

    def run_batch(self, mols: Sequence[atm.AtomList], defocus: Optional[Sequence[float]] = None) -> List:
        """Images of many molecules (optionally one defocus each), in input order."""
        m = self.microscope
        built = [self.build_slices(mol) for mol in mols]
        groups = defaultdict(list)
        for i, s in enumerate(built):
            groups[tuple(s.shape)].append(i)
        out: List = [None] * len(mols)
        for shape, idx in groups.items():
            stack = torch.stack([built[i] for i in idx])
            dfs = [m.defocus if defocus is None else defocus[i] for i in idx]
            wp = self._propagator(shape[-2:])
            imgs = wp.image(stack, self.slice_thickness, m.electron_dose, m.cs_mm, dfs, m.aperture)
            for j, i in enumerate(idx):
                out[i] = imgs[j]
        return out

    def __repr__(self):
        return (f"{{ImagePipe | resolution = {self._resolution}Angstrom, slice_thickness = {self.slice_thickness}"
                f"Angstrom, roi = {self.roi}, add_water = {self.add_water}, microscope = {self.microscope}}}")
