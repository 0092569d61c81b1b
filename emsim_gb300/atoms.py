"""Atom containers and the front-end geometry of the path (emsim/atoms.py:21-223,
emsim/utils/rot.py:8-157).

Coordinates are float32 with columns (z, x, y); slices run along column 0.  Every
operation keeps the reference's float32 evaluation order so that the binned
histograms are bit-identical.
"""
from __future__ import annotations

import bisect
import math
from typing import Generator, List, Optional, Sequence, Tuple, Union

import numpy as np

float_type = np.float32


class AtomList:
    """Elements (Z) and (N, 3) float32 coordinates (atoms.py:21-50)."""

    def __init__(self, elements: np.ndarray, coordinates: np.ndarray, label=""):
        self.elements = np.asarray(elements)
        # float32 as the reference stores them; no copy when they already are
        self.coordinates = np.asarray(coordinates).astype(float_type, copy=False)
        self.label = label

    @property
    def r_min(self):
        return self.coordinates.min(axis=0)

    @property
    def r_max(self):
        return self.coordinates.max(axis=0)

    @property
    def space(self):
        return self.r_max - self.r_min

    def __len__(self):
        return len(self.elements)

    def __repr__(self):
        return f"<AtomList consists of {len(self.elements)} atoms, label={self.label}>"


def sort_elements_and_count(atom_list: AtomList, must_include_elems: Optional[Sequence[int]] = ()):
    """Group atoms by Z; unique Z and counts, with zero counts for must-include Z
    (atoms.py:53-86).  Rows within an element keep numpy argsort order."""
    idx = np.argsort(atom_list.elements)
    elements = atom_list.elements[idx]
    coordinates = atom_list.coordinates[idx]
    unique_elements, counts = np.unique(elements, return_counts=True)
    for z in sorted(list(must_include_elems or ())):
        if z not in unique_elements:
            i = bisect.bisect_left(unique_elements, z)
            unique_elements = np.insert(unique_elements, i, z)
            counts = np.insert(counts, i, 0)
    return AtomList(elements=elements, coordinates=coordinates, label=atom_list.label), unique_elements, counts


def concatenate(atmls: List[AtomList]) -> AtomList:
    return AtomList(elements=np.concatenate([a.elements for a in atmls]),
                    coordinates=np.concatenate([a.coordinates for a in atmls]))


def translate(atom_list: AtomList, r) -> AtomList:
    return AtomList(elements=atom_list.elements, coordinates=atom_list.coordinates + r, label=atom_list.label)


def centralize(atom_list: AtomList) -> AtomList:
    """Origin at the bounding-box centre (atoms.py:142-159), float32 arithmetic."""
    return translate(atom_list, -atom_list.r_min - atom_list.space / 2.0)


def get_rotation_mattrices(quat: np.ndarray) -> np.ndarray:
    """Quaternions (B, 4) or (4,) -> (B, 3, 3) rotation matrices (utils/rot.py:107-157)."""
    quat = np.asarray(quat, dtype=np.float64)
    if quat.ndim == 1:
        quat = quat[None, :]
    elif quat.ndim > 2:
        raise ValueError("ndim of quat must be 1 or 2")
    if quat.shape[1] != 4:
        raise ValueError("quaternion must be 4D vector")
    q0, q1, q2, q3 = quat[:, 0], quat[:, 1], quat[:, 2], quat[:, 3]
    rot = np.empty((quat.shape[0], 3, 3), dtype=np.float64)
    rot[:, 0, 0] = 1. - 2. * (q2 * q2 + q3 * q3)
    rot[:, 0, 1] = 2. * (q1 * q2 + q0 * q3)
    rot[:, 0, 2] = 2. * (q1 * q3 - q0 * q2)
    rot[:, 1, 0] = 2. * (q1 * q2 - q0 * q3)
    rot[:, 1, 1] = 1. - 2. * (q1 * q1 + q3 * q3)
    rot[:, 1, 2] = 2. * (q0 * q1 + q2 * q3)
    rot[:, 2, 0] = 2. * (q0 * q2 + q1 * q3)
    rot[:, 2, 1] = 2. * (q2 * q3 - q0 * q1)
    rot[:, 2, 2] = 1. - 2. * (q1 * q1 + q2 * q2)
    return rot


def random_uniform_quaternions(n: int, rng: Optional[np.random.Generator] = None) -> np.ndarray:
    """Shoemake uniform random unit quaternions (utils/rot.py:8-53), (n, 4)."""
    rng = rng if rng is not None else np.random.default_rng()
    u1, u2, u3 = rng.random((3, n))
    return np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                     np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], axis=1)


def rotate(atom_list: AtomList, quat: np.ndarray, set_center: bool = False) -> AtomList:
    """Rotate by one quaternion (atoms.py:162-185)."""
    if set_center:
        atom_list = centralize(atom_list)
    rot = get_rotation_mattrices(quat)
    rot_coords = np.matmul(rot, atom_list.coordinates[..., None]).squeeze()
    return AtomList(elements=atom_list.elements, coordinates=rot_coords, label=atom_list.label)


def orientations_gen(atom_list: AtomList, quats: np.ndarray, set_center: bool = False) \
        -> Generator[AtomList, None, None]:
    for i in range(quats.shape[0]):
        yield rotate(atom_list, quats[i], set_center)


def determine_box_size(space: Tuple[float, float, float],
                       voxel_size: Union[float, Tuple[float, float, float]],
                       box_size: Tuple[Optional[int], Optional[int], Optional[int]]):
    """ceil(extent / voxel) per axis, 3.0 A for flat axes, overridden by box_size
    (atoms.py:214-223).  The division stays in float32 for float32 extents."""
    space = [3.0 if space[d] < 1e-3 else space[d] for d in range(3)]
    if type(voxel_size) is float:
        voxel_size = (voxel_size, voxel_size, voxel_size)
    box = [int(math.ceil(length / d)) for length, d in zip(space, voxel_size)]
    return tuple(box[d] if box_size[d] is None else box_size[d] for d in range(3))
