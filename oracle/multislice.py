"""numpy restatement of emsim's multislice hot path (test infrastructure only).

Every function cites the reference lines it restates (paths inside the emsim project).
Two semantics are provided, see ``oracle/__init__.py``:  ``"fftw"`` (FFTW/CUDA native
FP32 semantics; float32 = FP32 restatement, float64 = FP64 oracle) and ``"numpy"``
(numpy backend, complex128).

FFTs use ``scipy.fft`` so that float32 inputs are transformed in single precision (as
FFTW's ``fftwf_*`` and cuFFT do) and so that all host cores can be used
(``workers``).
"""
from __future__ import annotations

import math
import os
from fractions import Fraction
from pathlib import Path
from typing import Sequence, Tuple

import numpy as np
import scipy.fft as sfft

WORKERS = int(os.environ.get("EMSIM_ORACLE_WORKERS", "-1"))

# ---------------------------------------------------------------------------
# physics (emsim/physics.py:5-20 constants, 23-59, 62-81, 133-156)
# ---------------------------------------------------------------------------
E_STATC = 4.8032042510e-10
H_ERG_S = 6.62607015e-27
HBAR_ERG_S = H_ERG_S / 2.0 / math.pi
M0_G = 9.1093835611e-28
A0_CM = 5.29177210903e-9
C_CM_S = 29979245800.0
M0C2_ERG = M0_G * C_CM_S ** 2
HC_ERG_CM = H_ERG_S * C_CM_S
HBAR_C_ERG_CM = HBAR_ERG_S * C_CM_S
E_COULOMB = 1.602176634e-19
M0C2_KEV = M0C2_ERG * 1e-7 / E_COULOMB / 1000.
HC_KEV_ANG = HC_ERG_CM * 0.01 / E_COULOMB
WATER_NUM_DENS = 0.031


def wave_length(kev: float) -> float:
    """Relativistic electron wavelength in Angstrom (physics.py:44-59)."""
    return HC_KEV_ANG / math.sqrt(kev ** 2 + 2 * M0C2_KEV * kev)


def relativity_gamma(kev: float) -> float:
    """gamma = 1 + E/m0c^2 (physics.py:23-25)."""
    return 1 + kev / M0C2_KEV


def interaction_parameter(kev: float) -> float:
    """sigma in 1/(erg cm) units (physics.py:62-81)."""
    dimensionless = (M0C2_KEV + kev) / math.sqrt(kev * (2 * M0C2_KEV + kev))
    return (E_STATC / HBAR_C_ERG_CM) * dimensionless


def scherzer(wave_length_a: float, cs_mm: float) -> Tuple[float, float]:
    """Scherzer defocus (A) and aperture (rad) (physics.py:114-156)."""
    cslambda = cs_mm * 1e7 * wave_length_a
    df = math.sqrt((2 * 1 - 0.5) * cslambda)
    aper = pow(6 * wave_length_a / (cs_mm * 1e7), 0.25)
    return df, aper


# ---------------------------------------------------------------------------
# scattering factors (emsim/elem.py:120-156, 267-291, 294-354;
# emsim/backend/slice_builder_base.py:30-33)
# ---------------------------------------------------------------------------
_TABLE = Path(__file__).resolve().parent.parent / "emsim_gb300" / "data" / "kirkland_fe_params.csv"


def kirkland_params(zs: Sequence[int]) -> np.ndarray:
    """(len(zs), 12) float32 rows a1..a3, b1..b3, c1..c3, d1..d3."""
    tab = np.loadtxt(_TABLE, delimiter=",", comments="#", dtype=np.float64)
    out = []
    for z in zs:
        if not 1 <= int(z) <= 103:
            raise ValueError("z must be a interger in range [1, 92]")
        out.append(tab[int(z) - 1, 1:])
    return np.asarray(out, dtype=np.float32)


def scattering_factors2d(zs: Sequence[int], n1: int, n2: int, d1: float, d2: float) -> np.ndarray:
    """f_e on the fftshifted fftfreq grid, zero for q^2 >= 16; (nE, n1, n2) float32."""
    kx = np.fft.fftshift(np.fft.fftfreq(n1, d1))
    ky = np.fft.fftshift(np.fft.fftfreq(n2, d2))
    kx, ky = np.meshgrid(kx, ky, indexing="ij")
    k = np.sqrt(kx * kx + ky * ky)
    q2 = k * k
    mask = q2 < 16
    pms = kirkland_params(zs)
    out = np.empty((len(zs), n1, n2), dtype=np.float32)
    for e in range(len(zs)):
        a, b, c, d = pms[e, 0:3], pms[e, 3:6], pms[e, 6:9], pms[e, 9:12]
        v = np.sum([a[i] / (q2 + b[i]) + c[i] * np.exp(-d[i] * q2) for i in range(3)], axis=0)
        out[e] = np.where(mask, v, 0.)
    return out


def scattering_factors_half(zs: Sequence[int], n1: int, n2: int, d1: float, d2: float) -> np.ndarray:
    """Builder layout: ifftshifted, first n2//2+1 columns, float32 (nE, n1, n2//2+1)."""
    sf = scattering_factors2d(sorted(zs), n1, n2, d1, d2)
    sf = np.fft.ifftshift(sf, axes=(-2, -1))
    return np.ascontiguousarray(sf[:, :, :n2 // 2 + 1], dtype=np.float32)


# ---------------------------------------------------------------------------
# atoms front-end (emsim/atoms.py:53-86, 142-159, 162-185, 214-223; pot.py:51-74)
# ---------------------------------------------------------------------------
def sort_elements_and_count(elements: np.ndarray, coords: np.ndarray, must_include=()):
    idx = np.argsort(elements)
    el = elements[idx]
    xyz = coords.astype(np.float32)[idx]
    uz, cnt = np.unique(el, return_counts=True)
    for z in sorted(must_include):
        if z not in uz:
            i = int(np.searchsorted(uz, z))
            uz = np.insert(uz, i, z)
            cnt = np.insert(cnt, i, 0)
    return el, xyz, uz, cnt


def centralize(coords: np.ndarray) -> np.ndarray:
    c = coords.astype(np.float32)
    r_min = c.min(axis=0)
    space = c.max(axis=0) - r_min
    return c + (-r_min - space / 2.0)


def determine_box_size(space, voxel, box):
    space = [3.0 if space[d] < 1e-3 else space[d] for d in range(3)]
    b = [int(math.ceil(length / d)) for length, d in zip(space, voxel)]
    return tuple(b[d] if box[d] is None else box[d] for d in range(3))


def finalize_slice_size(space, pixel, thickness, lateral=None, n_slices=None):
    dims = [None, None, None]
    if lateral is not None:
        if isinstance(lateral, int):
            dims[1] = dims[2] = lateral
        else:
            dims[1], dims[2] = lateral
    if isinstance(n_slices, int):
        dims[0] = n_slices
    return determine_box_size(tuple(space), (thickness, pixel[0], pixel[1]), tuple(dims))


def rotation_matrix(quat: np.ndarray) -> np.ndarray:
    """Quaternion (q0,q1,q2,q3) -> 3x3 matrix, emsim/utils/rot.py:107-157 convention."""
    q0, q1, q2, q3 = [float(v) for v in quat]
    return np.array([
        [1. - 2. * (q2 * q2 + q3 * q3), 2. * (q1 * q2 + q0 * q3), 2. * (q1 * q3 - q0 * q2)],
        [2. * (q1 * q2 - q0 * q3), 1. - 2. * (q1 * q1 + q3 * q3), 2. * (q0 * q1 + q2 * q3)],
        [2. * (q0 * q2 + q1 * q3), 2. * (q2 * q3 - q0 * q1), 1. - 2. * (q1 * q1 + q2 * q2)]])


# ---------------------------------------------------------------------------
# binning
# ---------------------------------------------------------------------------
def _f32_round(fr: Fraction) -> np.float32:
    """Correctly rounded float32 of an exact rational (round half to even)."""
    if fr == 0:
        return np.float32(0.0)
    sign = -1 if fr < 0 else 1
    a = abs(fr)
    e = a.numerator.bit_length() - a.denominator.bit_length()
    if Fraction(2) ** e > a:
        e -= 1
    e = max(e, -126)
    scale = Fraction(2) ** (e - 23)
    m = a / scale
    q = m.numerator // m.denominator
    rem = m - q
    if rem > Fraction(1, 2) or (rem == Fraction(1, 2) and q % 2 == 1):
        q += 1
    return np.float32(sign * float(q * scale))


def cuda_bin_edges(n: int, d: float) -> Tuple[np.float32, np.float32, np.float32]:
    """Start/end edge of the CUDA rule (SliceBuilder_kernel.cu:30-34, 87-92).

    start = -d * floorf((float)(n+1)/2.0f) in float32; end = start + (float)n * d,
    which nvcc contracts into one fused multiply-add (single rounding).
    """
    d32 = np.float32(d)
    half = np.float32(math.floor(np.float32(n + 1) / np.float32(2.0)))
    start = np.float32(-(d32 * half))
    end = _f32_round(Fraction(n) * Fraction(float(d32)) + Fraction(float(start)))
    return d32, start, end


def _cuda_axis_index(x: np.ndarray, n: int, d: float):
    """Bin index + inside mask for one axis with the CUDA rule (SliceBuilder_kernel.cu:52-55).

    Inside: start <= x <= end.  Index: n-1 when (end - x) < 1e-12 (float difference
    compared in double, the LEFT_CLOSE macro), else floorf((x - start) / d).  An index
    that rounds up to n (x a hair below end) is clamped to n-1; the reference writes
    out of bounds there.
    """
    d32, start, end = cuda_bin_edges(n, d)
    x = x.astype(np.float32)
    inside = (start <= x) & (x <= end)
    diff = (end - x).astype(np.float32).astype(np.float64)
    idx = np.floor((x - start) / d32).astype(np.float64)
    idx = np.where(diff < 1e-12, n - 1, idx)
    idx = np.clip(idx, 0, n - 1)
    return idx.astype(np.int64), inside


def _element_of_rows(counts: np.ndarray, n_atoms: int) -> np.ndarray:
    """Element index of each row from the per-element counts (SliceBuilder_kernel.cu:44-48).

    A row past sum(counts) falls to element nE-1... the reference loop leaves e == nElems,
    which indexes past the output; such rows are rejected here (never produced by
    sort_elements_and_count)."""
    bounds = np.cumsum(np.asarray(counts, dtype=np.int64))
    return np.searchsorted(bounds, np.arange(n_atoms), side="right")


def bin_atoms_cuda(coords: np.ndarray, counts: np.ndarray, shape: Tuple[int, ...],
                   steps: Tuple[float, ...]) -> np.ndarray:
    """CUDA-rule histogram (SliceBuilder_kernel.cu:9-61 one slice, 64-123 multi slice).

    ``shape``/``steps`` of length 2 -> (n1, n2) using coordinate columns 1, 2;
    length 3 -> (n0, n1, n2) using columns 0, 1, 2.  Returns float32 (nE, *shape).
    """
    coords = np.asarray(coords, dtype=np.float32).reshape(-1, 3)
    n_atoms = coords.shape[0]
    n_elems = len(counts)
    cols = (1, 2) if len(shape) == 2 else (0, 1, 2)
    elem = _element_of_rows(counts, n_atoms)
    keep = elem < n_elems
    lin = elem.astype(np.int64)
    for ax, (col, n, d) in enumerate(zip(cols, shape, steps)):
        idx, inside = _cuda_axis_index(coords[:, col], n, d)
        keep &= inside
        lin = lin * n + idx
    out = np.zeros((n_elems,) + tuple(shape), dtype=np.float32)
    flat = np.bincount(lin[keep], minlength=out.size).astype(np.float32)
    return flat.reshape(out.shape)


def numpy_bin_edges(n: int, d: float) -> np.ndarray:
    """slice_builder_base.py:183-185 edges: arange(start, end + d, d), start = -d*(n//2)."""
    start = -d * (n // 2)
    end = start + n * d
    return np.arange(start, end + d, d)


def bin_atoms_numpy(coords: np.ndarray, counts: np.ndarray, shape: Tuple[int, ...],
                    steps: Tuple[float, ...]) -> np.ndarray:
    """numpy-rule histogram (slice_builder_base.py:180-225): histogramdd over arange edges.

    The bin count per axis is len(edges)-1, which equals n except when arange's float
    end-point rounding adds an edge; the reference returns that shape as is.
    """
    coords = np.asarray(coords)
    cols = (1, 2) if len(shape) == 2 else (0, 1, 2)
    edges = [numpy_bin_edges(n, d) for n, d in zip(shape, steps)]
    nb = [len(e) - 1 for e in edges]
    out = np.empty((len(counts), *nb), dtype=np.float32)
    m = 0
    for i, n in enumerate(counts):
        n = int(n)
        if n == 0:
            out[i] = 0
        else:
            pts = coords[m:m + n][:, cols]
            out[i], _ = np.histogramdd(pts, bins=edges)
        m += n
    return np.ascontiguousarray(out, dtype=np.float32)


# ---------------------------------------------------------------------------
# projected-potential slices
# ---------------------------------------------------------------------------
def bandlimit_mask_half(n1: int, n2: int) -> np.ndarray:
    """Circular band-limit of radius min(n1,n2)//2 on the centred integer grid,
    ifftshifted, first n2//2+1 columns (slice_builder_cuda.py:88-99,
    slice_builder_base.py:166-175).  The reference builds it with 'xy' meshgrid, which
    only has a consistent shape for n1 == n2; this builds the intended (n1, n2) mask."""
    r = min(n1, n2) // 2
    k1 = np.arange(-n1 // 2, -n1 // 2 + n1)
    k2 = np.arange(-n2 // 2, -n2 // 2 + n2)
    kk1, kk2 = np.meshgrid(k1, k2, indexing="ij")
    fil = (kk1 ** 2 + kk2 ** 2 <= r ** 2).astype(np.float32)
    fil = np.fft.ifftshift(fil)
    return np.ascontiguousarray(fil[:, :n2 // 2 + 1])


def make_slices(hist: np.ndarray, sf_half: np.ndarray, semantics: str = "fftw",
                dtype=np.float32, bandlimit: bool = True) -> np.ndarray:
    """Projected-potential slices from element histograms.

    hist: (nE, nS, n1, n2) or (nE, n1, n2); sf_half: (nE, n1, n2//2+1).
    ``fftw``: R2C per (element, slice), multiply by SF and 1/N, accumulate over elements
    in order, C2R unnormalised (SliceBuilder.cpp:27-85 / SliceBuilder.cu:108-133), then
    the float32 band-limit round trip (slice_builder_cuda.py:88-99) and the clip at 1e-13.
    ``numpy``: slice_builder_numpy.py:18-26, 37-44 verbatim in numpy.
    """
    one = hist.ndim == 3
    h = hist[:, None] if one else hist
    n1, n2 = h.shape[-2:]
    if semantics == "numpy":
        lp = np.fft.rfft2(h, axes=(-2, -1))
        lp *= sf_half[:, None, :, :]
        s = np.fft.irfft2(np.sum(lp, axis=0), s=(n1, n2))
        if bandlimit:
            r = min(n1, n2) // 2
            kx, ky = np.meshgrid(np.arange(-n1 // 2, -n1 // 2 + n1), np.arange(-n2 // 2, -n2 // 2 + n2))
            fil = np.fft.ifftshift(np.where(kx ** 2 + ky ** 2 <= r ** 2, 1, 0))
            ft = np.fft.rfft2(s, axes=(-2, -1), s=(n1, n2))
            s = np.fft.irfft2(ft * fil[:, :n2 // 2 + 1], s=(n1, n2))
        np.clip(s, a_min=1e-13, a_max=None, out=s)
        return s[0] if one else s
    rdt = np.dtype(dtype)
    cdt = np.complex64 if rdt == np.float32 else np.complex128
    npix = rdt.type(n1 * n2)
    H = sfft.rfft2(h.astype(rdt), axes=(-2, -1), workers=WORKERS).astype(cdt)
    acc = np.zeros(H.shape[1:], dtype=cdt)
    for k in range(H.shape[0]):
        acc += H[k] * sf_half[k].astype(rdt)
    acc = (acc.real / npix + 1j * (acc.imag / npix)).astype(cdt)
    s = sfft.irfft2(acc, s=(n1, n2), axes=(-2, -1), norm="forward", workers=WORKERS).astype(rdt)
    if bandlimit:
        fil = bandlimit_mask_half(n1, n2).astype(rdt)
        ft = sfft.rfft2(s, axes=(-2, -1), workers=WORKERS).astype(cdt)
        s = sfft.irfft2(ft * fil, s=(n1, n2), axes=(-2, -1), workers=WORKERS).astype(rdt)
    s = np.clip(s, rdt.type(1e-13), None).astype(rdt)
    return s[0] if one else s


# ---------------------------------------------------------------------------
# wave propagation
# ---------------------------------------------------------------------------
PI32 = np.float32(3.14159265358979324)


def fftw_freq_sq(n1: int, n2: int, d1: float, d2: float, dtype=np.float32) -> np.ndarray:
    """|f|^2 on the unshifted FFT grid with the reference's index arithmetic
    (WavePropagator.cpp:19-21, 63-71; WavePropagator_kernel.cu:53-79): dfx = 1/d1/n1,
    fx = (is - floor(n1/2)) * dfx where is - floor(n1/2) is the fftfreq integer.
    float32 evaluates without fused multiply-add, as the C++ extension does."""
    t = np.dtype(dtype).type
    dfx = t(1.0) / t(d1) / t(n1)
    dfy = t(1.0) / t(d2) / t(n2)
    i = np.arange(n1)
    j = np.arange(n2)
    ki = np.where(i < (n1 + 1) // 2, i, i - n1).astype(dtype)
    kj = np.where(j < (n2 + 1) // 2, j, j - n2).astype(dtype)
    fx = (ki * dfx).astype(dtype)
    fy = (kj * dfy).astype(dtype)
    return (fx[:, None] * fx[:, None]).astype(dtype) + (fy[None, :] * fy[None, :]).astype(dtype)


def numpy_q_grid(n1: int, n2: int, d1: float, d2: float) -> np.ndarray:
    """|q| on the linspace grid of wave_propagator_base.py:47-53 (fftshifted layout)."""
    qx = np.linspace(-0.5 / d1, 0.5 / d1, n1)
    qy = np.linspace(-0.5 / d2, 0.5 / d2, n2)
    qx, qy = np.meshgrid(qx, qy, indexing="ij")
    return np.sqrt(qx * qx + qy * qy)


class WavePropagator:
    """Restatement of the reference WavePropagator for one (n1, n2, d1, d2, kV).

    fftw semantics: WavePropagator.cpp:15-138 / WavePropagator.cu + _kernel.cu.
    numpy semantics: wave_propagator_base.py:11-53 + wave_propagator_numpy.py:18-47.
    """

    def __init__(self, n1: int, n2: int, d1: float, d2: float, beam_energy_kev: float,
                 semantics: str = "fftw", dtype=np.float32):
        self.n1, self.n2, self.d1, self.d2 = n1, n2, d1, d2
        self.semantics = semantics
        self.rdt = np.dtype(dtype)
        self.cdt = np.complex64 if self.rdt == np.float32 else np.complex128
        self.wave_length = wave_length(beam_energy_kev)
        self.relativity_gamma = relativity_gamma(beam_energy_kev)
        if semantics == "numpy":
            self.q = numpy_q_grid(n1, n2, d1, d2)
            q_max = 0.5 / max(d1, d2)
            self.fil = np.fft.ifftshift(np.where(self.q <= q_max * 0.6667, 1., 0.))
        else:
            t = self.rdt.type
            self.f2 = fftw_freq_sq(n1, n2, d1, d2, self.rdt)
            fmax = t(0.5) / t(max(d1, d2))
            self.filt = t(0.6667) * fmax
            self.lam = t(self.wave_length)
            self.gam = t(self.relativity_gamma)
            self.pi = PI32 if self.rdt == np.float32 else np.float64(math.pi)

    # -- helpers ------------------------------------------------------------
    def _fft2(self, w):
        return sfft.fft2(w.astype(self.cdt), workers=WORKERS)

    def _ifft2_unnorm(self, w):
        return sfft.ifft2(w, norm="forward", workers=WORKERS)

    def _cmul(self, w, pr, pi):
        """(w.re + i w.im)(pr + i pi) with separate real products, no FMA."""
        t = self.rdt
        re = (w.real * pr).astype(t) - (w.imag * pi).astype(t)
        im = (w.real * pi).astype(t) + (w.imag * pr).astype(t)
        return (re + 1j * im).astype(self.cdt)

    # -- API ------------------------------------------------------------------
    def init_wave(self, dose: float) -> np.ndarray:
        """wave_propagator_base.py:25-29: complex64 sqrt(dose*d1*d2) everywhere."""
        n_e = dose * self.d1 * self.d2
        w = np.ones((self.n1, self.n2), dtype=np.complex64)
        w *= np.sqrt(n_e) / np.abs(w)
        return w

    def slice_transmit(self, wave, aslice):
        if self.semantics == "numpy":
            return wave * np.exp(1j * self.relativity_gamma * self.wave_length * aslice)
        t = self.rdt.type
        factor = t(self.lam * self.gam)
        ph = (np.asarray(aslice).astype(self.rdt) * factor).astype(self.rdt)
        return self._cmul(np.asarray(wave).astype(self.cdt), np.cos(ph), np.sin(ph))

    def _propagator(self, dz: float):
        t = self.rdt.type
        ph = (((self.lam * self.pi).astype(self.rdt) * t(dz)).astype(self.rdt) * self.f2).astype(self.rdt)
        keep = self.f2 <= (self.filt * self.filt)
        return np.cos(ph), -np.sin(ph), keep

    def space_propagate(self, wave, dz: float):
        if self.semantics == "numpy":
            p = np.exp(-1j * self.wave_length * np.pi * dz * self.q ** 2)
            return np.fft.ifft2(np.fft.ifftshift(p) * np.fft.fft2(wave))
        F = self._fft2(wave)
        pr, pi, keep = self._propagator(dz)
        t = self.rdt.type
        n = t(self.n1 * self.n2)
        G = self._cmul(F, pr, pi)
        G = ((G.real / n) + 1j * (G.imag / n)).astype(self.cdt)
        G[~keep] = 0
        return self._ifft2_unnorm(G).astype(self.cdt)

    def singleslice_propagate(self, wave, aslice, dz: float):
        if self.semantics == "numpy":
            p = np.exp(-1j * self.wave_length * np.pi * dz * self.q ** 2)
            tr = np.exp(1j * self.relativity_gamma * self.wave_length * aslice)
            return np.fft.ifft2(np.fft.ifftshift(p) * np.fft.fft2(wave * tr) * self.fil)
        return self.space_propagate(self.slice_transmit(wave, aslice), dz)

    def multislice_propagate(self, wave, slices, dz: float):
        if self.semantics == "numpy":
            p = np.exp(-1j * self.wave_length * np.pi * dz * self.q ** 2)
            tr = np.exp(1j * self.relativity_gamma * self.wave_length * slices)
            psi = wave
            for s in range(slices.shape[0]):
                psi = np.fft.ifft2(np.fft.ifftshift(p) * np.fft.fft2(psi * tr[s]) * self.fil)
            return psi
        psi = np.asarray(wave).astype(self.cdt)
        for s in range(slices.shape[0]):
            psi = self.singleslice_propagate(psi, slices[s], dz)
        return psi

    def lens_transfer(self, cs_mm: float, defocus: float, aperture: float):
        """(h_re, h_im, keep) of WavePropagator.cpp:105-138 on the unshifted grid."""
        t = self.rdt.type
        lam, pi = self.lam, self.pi
        c1 = t(t(t(t(t(t(0.5) * pi) * t(cs_mm)) * t(1e7)) * lam) * lam) * lam
        c2 = t(t(pi * t(defocus)) * lam)
        f_aper = t(aperture) / lam
        f2 = self.f2
        keep = f2 <= f_aper * f_aper
        ab = ((c1 * f2).astype(self.rdt) * f2).astype(self.rdt) - (c2 * f2).astype(self.rdt)
        ab = ab.astype(self.rdt)
        return np.cos(ab), -np.sin(ab), keep

    def lens_propagate(self, wave, cs_mm: float, defocus: float, aperture: float):
        if self.semantics == "numpy":
            lam = self.wave_length
            cslambda = cs_mm * 1e7 * lam
            D = defocus / math.sqrt(cslambda)
            K = self.q * pow(cslambda * lam ** 2, 0.25)
            chi = math.pi * (0.5 * K ** 4 - D * K ** 2)
            h = np.exp(-1j * chi)
            h *= np.where(self.q < aperture / lam, 1., 0.)
            return np.fft.ifft2(np.fft.ifftshift(h) * np.fft.fft2(wave))
        F = self._fft2(wave)
        hr, hi, keep = self.lens_transfer(cs_mm, defocus, aperture)
        n = self.rdt.type(self.n1 * self.n2)
        G = self._cmul(F, hr, hi)
        G = ((G.real / n) + 1j * (G.imag / n)).astype(self.cdt)
        G[~keep] = 0
        return self._ifft2_unnorm(G).astype(self.cdt)


def band_limit_slices(slices: np.ndarray) -> np.ndarray:
    """tem.band_limit_specimen (tem.py:102-108) as intended: every (n1, n2) slice of a
    (n_slices, n1, n2) stack is low-passed with the disc (x - n1//2)^2 + (y - n2//2)^2 <=
    4 r^2 / 9 (r = min(n1, n2)//2) on the centred grid, ifftshifted, real part kept
    (complex128).  The reference's own code transforms axes (0, 1) of the array it is
    given, so it agrees with this for a stack transposed to (n1, n2, n_slices) with
    n2 == n_slices, e.g. a cubic one."""
    s = np.asarray(slices, dtype=np.float64)
    n1, n2 = s.shape[-2:]
    r = min(n1, n2) // 2
    x, y = np.mgrid[0:n1, 0:n2]
    fil = np.fft.ifftshift(np.where((x - n1 // 2) ** 2 + (y - n2 // 2) ** 2 <= 4 * r * r / 9, 1., 0.))
    return np.fft.ifft2(np.fft.fft2(s, axes=(-2, -1)) * fil, axes=(-2, -1)).real


def intensity(wave: np.ndarray) -> np.ndarray:
    """pipe.py:81-82: re^2 + im^2."""
    return wave.real ** 2 + wave.imag ** 2


# ---------------------------------------------------------------------------
# end-to-end pipeline (emsim/pipe.py:46-84 with pot.py:29-48)
# ---------------------------------------------------------------------------
def build_multi_slices(elements, coords, dz, pixel, lateral=None, n_slices=None,
                       semantics="fftw", dtype=np.float32, return_hist=False):
    """pot.build_multi_slices (pot.py:29-48) without water."""
    if isinstance(pixel, (int, float)):
        pixel = (float(pixel), float(pixel))
    el, xyz, uz, cnt = sort_elements_and_count(np.asarray(elements), np.asarray(coords))
    space = xyz.max(axis=0) - xyz.min(axis=0)
    ns, n1, n2 = finalize_slice_size(space, pixel, dz, lateral, n_slices)
    if semantics == "numpy":
        hist = bin_atoms_numpy(xyz, cnt, (ns, n1, n2), (dz, pixel[0], pixel[1]))
    else:
        hist = bin_atoms_cuda(xyz, cnt, (ns, n1, n2), (dz, pixel[0], pixel[1]))
    sf = scattering_factors_half(list(uz), n1, n2, pixel[0], pixel[1])
    slices = make_slices(hist, sf, semantics, dtype)
    if return_hist:
        return slices, hist
    return slices


def pipe_run(elements, coords, *, resolution, slice_thickness, roi, beam_energy_kev, dose,
             cs_mm, defocus, aperture, semantics="fftw", dtype=np.float32, n_slices=None,
             return_exit_wave=False):
    """Pipe.run (pipe.py:46-55, 79-84) with add_water=False.  ``n_slices`` is honoured
    here (the reference's Pipe drops it, pipe.py:48-52; pass None for that behaviour)."""
    pixel = 0.5 * resolution
    xyz = centralize(np.asarray(coords))
    slices = build_multi_slices(elements, xyz, slice_thickness, pixel, roi, n_slices, semantics, dtype)
    roi2 = (roi, roi) if isinstance(roi, int) else roi
    wp = WavePropagator(roi2[0], roi2[1], pixel, pixel, beam_energy_kev, semantics, dtype)
    w0 = wp.init_wave(dose)
    ew = wp.multislice_propagate(w0, slices, slice_thickness)
    iw = wp.lens_propagate(ew, cs_mm, defocus, aperture)
    img = intensity(iw)
    if return_exit_wave:
        return img, ew
    return img


# ---------------------------------------------------------------------------
# seeded synthetic inputs (workloads named by their sizes)
# ---------------------------------------------------------------------------
def five_atoms():
    """Z = 6, 14, 29, 79, 92 on the z = 0 plane at y = 5..45 A (demos/five_atoms.py:17-22)."""
    el = np.array([6, 14, 29, 79, 92])
    xyz = np.array([[0, 0, 5], [0, 0, 15], [0, 0, 25], [0, 0, 35], [0, 0, 45]], dtype=np.float32)
    return el, centralize(xyz)


def protein_blob(n_atoms: int = 50_000, radius: float = 40.0, seed: int = 0):
    """C/N/O/S (0.63/0.17/0.19/0.01) uniform in a ball, seeded; float32 (z, x, y)."""
    rng = np.random.default_rng(seed)
    el = rng.choice(np.array([6, 7, 8, 16]), size=n_atoms, p=[0.63, 0.17, 0.19, 0.01])
    v = rng.normal(size=(n_atoms, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    r = radius * rng.random(n_atoms) ** (1.0 / 3.0)
    return el, (v * r[:, None]).astype(np.float32)


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.complex128)
    b = np.asarray(b, dtype=np.complex128)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
