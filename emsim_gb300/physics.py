"""Electron-optics constants and formulas in FP64 (emsim/physics.py:5-156).

Same CODATA constants and the same formula order as the reference, so wavelength,
relativistic gamma, interaction parameter and Scherzer conditions are bit-identical.
"""
import math

import numpy as np

water_num_dens = 0.031  # molecules per A^3
e = 4.8032042510e-10  # statC
h = 6.62607015e-27  # erg s
hbar = h / 2.0 / math.pi
m0 = 9.1093835611e-28  # g
a0 = 5.29177210903e-9  # cm
c = 29979245800.0  # cm / s
m0c2 = m0 * c ** 2
hc = h * c
hbar_c = hbar * c
e_coulumb = 1.602176634e-19
m0c2_keV = m0c2 * 1e-7 / e_coulumb / 1000.
hbar_c_keV_Ang = hbar_c * 0.01 / e_coulumb
hc_keV_Ang = hc * 0.01 / e_coulumb


def electron_relativity_gamma(beam_energy_kev: float) -> float:
    return 1 + beam_energy_kev / m0c2_keV


def electron_wave_length_angstrom(beam_energy_kev: float) -> float:
    return hc_keV_Ang / math.sqrt(beam_energy_kev ** 2 + 2 * m0c2_keV * beam_energy_kev)


def interaction_parameter(beam_energy_kev: float) -> float:
    dimensionless = (m0c2_keV + beam_energy_kev) / math.sqrt(beam_energy_kev * (2 * m0c2_keV + beam_energy_kev))
    return (e / hbar_c) * dimensionless


def aberration(wave_length_angstrom: float, cs_mm: float, defocus_angstrom: float):
    cslambda = cs_mm * 1e7 * wave_length_angstrom
    D = defocus_angstrom / math.sqrt(cslambda)

    def aberration_(k):
        K = k * pow(cslambda * wave_length_angstrom ** 2, 0.25)
        return math.pi * (0.5 * K ** 4 - D * K ** 2)
    return aberration_


def mtf(wave_length_angstrom: float, cs_mm: float, defocus_angstrom: float):
    def mtf_(k):
        return np.exp(-1j * aberration(wave_length_angstrom, cs_mm, defocus_angstrom)(k))
    return mtf_


def ctf(wave_length_angstrom: float, cs_mm: float, defocus_angstrom: float):
    def ctf_(k):
        return np.sin(aberration(wave_length_angstrom, cs_mm, defocus_angstrom)(k))
    return ctf_


def optimal_focus(wave_length_angstrom: float, cs_mm: float, nd: int) -> float:
    cslambda = cs_mm * 1e7 * wave_length_angstrom
    return math.sqrt((2 * nd - 0.5) * cslambda)


def scherzer_condition(wave_length_angstrom: float, cs_mm: float):
    df = optimal_focus(wave_length_angstrom, cs_mm, 1)
    aper = pow(6 * wave_length_angstrom / (cs_mm * 1e7), 0.25)
    return df, aper
