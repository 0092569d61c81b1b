"""Differentiable image formation: intensity = |lens(multislice(plane wave, slices))|^2
with the gradient of a loss with respect to the slice potentials, and off-grid slices
with the gradient with respect to the atom coordinates.

emsim forms images without derivatives (pipe.py:46-55, 79-84); this module puts the
engine's checkpointed forward (``emsim_gb300_multislice_image_ckpt``) and adjoint
multislice (``emsim_gb300_multislice_image_adjoint``) behind a
``torch.autograd.Function``.  The forward keeps the complex image wave and one wave
state every ``every`` slices (default ceil(sqrt(n_slices))); the backward recomputes one
segment of transmitted waves at a time and runs the conjugate steps.  Slices shared by a
batch of images (one stack, several defocus values) receive the sum of the images'
gradients, added in image order.
"""
from __future__ import annotations

import ctypes
import math
from typing import Optional, Sequence, Union

import numpy as np
import torch

from . import _native
from .backend import MultiSlicesBuilder, WavePropagator, _ptr, _stream

__all__ = ["MultisliceImage", "image", "default_every", "SmoothSlices", "smooth_slices"]


def default_every(n_slices: int) -> int:
    """Checkpoint spacing giving O(sqrt(n_slices)) stored waves."""
    return max(1, int(math.ceil(math.sqrt(max(1, n_slices)))))


def _defocus_array(defocus) -> np.ndarray:
    return np.ascontiguousarray(np.atleast_1d(np.asarray(defocus, dtype=np.float64)))


class MultisliceImage(torch.autograd.Function):
    """images (nb, n1, n2) float32 = |L P t_{S-1} ... P t_0 psi_0|^2 for slices of shape
    (S, n1, n2) (shared by nb images) or (nb, S, n1, n2)."""

    @staticmethod
    def forward(ctx, slices: torch.Tensor, wp: WavePropagator, dz: float, dose: float, cs_mm: float,
                defocus: np.ndarray, aperture: float, nb: int, every: int):
        n1, n2 = wp.wave_shape
        s = slices.detach()
        if s.dtype != torch.float32 or not s.is_cuda:
            raise TypeError("slices must be a float32 CUDA tensor")
        s = s.contiguous()
        if s.dim() == 4:
            ns, stride = int(s.shape[1]), int(s.shape[1]) * n1 * n2
        else:
            ns, stride = int(s.shape[0]), 0
        lib = _native.load()
        n_ck = int(lib.emsim_gb300_adjoint_checkpoints(ns, every))
        img = torch.empty((nb, n1, n2), dtype=torch.float32, device=s.device)
        u = torch.empty((nb, n1, n2), dtype=torch.complex64, device=s.device)
        ck = torch.empty((max(n_ck, 0), nb, n1, n2), dtype=torch.complex64, device=s.device)
        dfp = defocus.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        _native.call("emsim_gb300_multislice_image_ckpt", wp._plan.handle, _ptr(s), ns, stride, float(dz),
                     float(dose), float(cs_mm), dfp, len(defocus), float(aperture), _ptr(img), _ptr(u),
                     _ptr(ck) if n_ck > 0 else None, every, nb, _stream())
        ctx.save_for_backward(s, u, ck)
        ctx.params = (wp, float(dz), float(dose), float(cs_mm), defocus, float(aperture), nb, every, ns, stride)
        return img

    @staticmethod
    def backward(ctx, grad_image: torch.Tensor):
        s, u, ck = ctx.saved_tensors
        wp, dz, dose, cs_mm, defocus, aperture, nb, every, ns, stride = ctx.params
        g = grad_image.detach().to(torch.float32).contiguous()
        lib = _native.load()
        nbytes = int(lib.emsim_gb300_adjoint_workspace_size(wp._plan.handle, ns, every, nb, stride))
        work = torch.empty(nbytes, dtype=torch.uint8, device=s.device)
        grad = torch.empty_like(s)
        dfp = defocus.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
        _native.call("emsim_gb300_multislice_image_adjoint", wp._plan.handle, _ptr(s), ns, stride, dz, dose, cs_mm,
                     dfp, len(defocus), aperture, _ptr(g), _ptr(u), _ptr(ck) if ck.numel() else None, every,
                     _ptr(grad), _ptr(work), nbytes, nb, _stream())
        return grad, None, None, None, None, None, None, None, None


def image(wp: WavePropagator, slices: torch.Tensor, dz: float, electron_dose: float, cs_mm: float,
          defocus: Union[float, Sequence[float]], aperture: float, n_batch: Optional[int] = None,
          every: Optional[int] = None) -> torch.Tensor:
    """Differentiable ``WavePropagator.image``: (nb, n1, n2) float32 intensities.

    ``slices``: float32 CUDA tensor (S, n1, n2) shared by the batch or (nb, S, n1, n2);
    ``defocus``: a number or a sequence (image b uses defocus[b % len]); ``n_batch``
    defaults to len(defocus) for shared slices; ``every``: checkpoint spacing."""
    dfs = _defocus_array(defocus)
    if slices.dim() == 4:
        nb = int(slices.shape[0])
        ns = int(slices.shape[1])
    elif slices.dim() == 3:
        nb = int(n_batch or len(dfs))
        ns = int(slices.shape[0])
    else:
        raise ValueError("slices must be (S, n1, n2) or (nb, S, n1, n2)")
    if tuple(slices.shape[-2:]) != tuple(wp.wave_shape):
        raise ValueError(f"slices of shape {tuple(slices.shape)} do not match the wave {wp.wave_shape}")
    ev = int(every) if every else default_every(ns)
    return MultisliceImage.apply(slices, wp, float(dz), float(electron_dose), float(cs_mm), dfs, float(aperture), nb,
                                 ev)


class SmoothSlices(torch.autograd.Function):
    """Off-grid slices (``emsim_gb300_build_slices_smooth``) of molecules given as
    coordinates sorted by element; the backward returns dLoss/dcoords (z column 0)."""

    @staticmethod
    def forward(ctx, coords: torch.Tensor, builder: MultiSlicesBuilder, counts: torch.Tensor, nb: int):
        c = coords.detach()
        if c.dtype != torch.float32 or not c.is_cuda:
            raise TypeError("coords must be a float32 CUDA tensor")
        c = c.contiguous()
        n_atoms = int(c.shape[0])
        plan = builder._plan.handle
        lib = _native.load()
        nbytes = int(lib.emsim_gb300_smooth_workspace_size(plan, n_atoms, nb))
        ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=c.device)
        out = torch.empty((nb, builder.n_slice, builder.n1, builder.n2), dtype=torch.float32, device=c.device)
        _native.call("emsim_gb300_build_slices_smooth", plan, _ptr(c), n_atoms, _ptr(counts), nb, _ptr(out), _ptr(ws),
                     nbytes, _stream())
        ctx.save_for_backward(c, counts, out)
        ctx.builder, ctx.nb = builder, nb
        return out

    @staticmethod
    def backward(ctx, grad_slices: torch.Tensor):
        c, counts, out = ctx.saved_tensors
        builder, nb = ctx.builder, ctx.nb
        n_atoms = int(c.shape[0])
        plan = builder._plan.handle
        lib = _native.load()
        nbytes = int(lib.emsim_gb300_smooth_workspace_size(plan, n_atoms, nb))
        ws = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=c.device)
        g = grad_slices.detach().to(torch.float32).contiguous()
        grad = torch.zeros_like(c)
        _native.call("emsim_gb300_build_slices_smooth_adjoint", plan, _ptr(c), n_atoms, _ptr(counts), nb, _ptr(out),
                     _ptr(g), _ptr(grad), _ptr(ws), nbytes, _stream())
        return grad, None, None, None


def smooth_slices(builder: MultiSlicesBuilder, coords: torch.Tensor, elem_counts) -> torch.Tensor:
    """Differentiable off-grid slices.  ``coords``: (N, 3) float32 CUDA tensor (columns
    z, x, y), molecules back to back, each sorted by element; ``elem_counts``: (nE,) for
    one molecule -> (n_slices, n1, n2), or (B, nE) -> (B, n_slices, n1, n2), counts in
    the builder's element order."""
    cnt = np.ascontiguousarray(np.asarray(elem_counts, dtype=np.uint32))
    one = cnt.ndim == 1
    cnt2 = cnt.reshape(1, -1) if one else cnt
    if cnt2.shape[1] != len(builder.unique_elements):
        raise ValueError(f"elem_counts must have {len(builder.unique_elements)} entries per molecule")
    counts = torch.as_tensor(cnt2.view(np.int32), device=coords.device).contiguous()
    out = SmoothSlices.apply(coords, builder, counts, int(cnt2.shape[0]))
    return out[0] if one else out
