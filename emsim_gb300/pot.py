"""Projected-potential front-end (emsim/pot.py:13-74) on the GB300 backend."""
from __future__ import annotations

from typing import Optional, Tuple, Union

from . import atoms as atm
from . import backend


def finalize_slice_size(mol_space, pixel_size, thickness: float,
                        lateral_size: Optional[Union[int, Tuple[int, int]]] = None,
                        n_slices: Optional[int] = None):
    """(n_slices, n1, n2) from the extent, overridden by lateral_size / n_slices (pot.py:51-74)."""
    dims = [None, None, None]
    if lateral_size is not None:
        if isinstance(lateral_size, int):
            dims[1] = dims[2] = lateral_size
        elif isinstance(lateral_size, tuple) and len(lateral_size) == 2:
            dims[1], dims[2] = lateral_size
    if isinstance(n_slices, int):
        dims[0] = n_slices
    if isinstance(pixel_size, float):
        pixel_size = (pixel_size, pixel_size)
    return atm.determine_box_size(tuple(mol_space), voxel_size=(thickness, pixel_size[0], pixel_size[1]),
                                  box_size=(dims[0], dims[1], dims[2]))


def build_one_slice(mol: atm.AtomList, pixel_size: Union[float, Tuple[float, float]],
                    lateral_size: Optional[Union[int, Tuple[int, int]]] = None):
    """pot.py:13-26: sort by element, size the grid (thickness 5 A), bin, build."""
    if type(pixel_size) is float:
        pixel_size = (pixel_size,) * 2
    mol, uz, cnt = atm.sort_elements_and_count(mol)
    _, n1, n2 = finalize_slice_size(tuple(mol.space), pixel_size, 5.0, lateral_size, 1)
    b = backend.OneSliceBuilder(list(uz), n1, n2, pixel_size[0], pixel_size[1])
    return b.make_one_slice(b.bin_atoms_one_slice(mol.coordinates, cnt))


def build_multi_slices(mol: atm.AtomList, dz: float, pixel_size: Union[float, Tuple[float, float]],
                       lateral_size: Optional[Union[int, Tuple[int, int]]] = None,
                       n_slices: Optional[int] = None, add_water: bool = False):
    """pot.py:29-48: sort (with H and O when adding water), size, bin, [water], build."""
    if type(pixel_size) is float:
        pixel_size = (pixel_size,) * 2
    must = [1, 8] if add_water else []
    mol, uz, cnt = atm.sort_elements_and_count(mol, must)
    ns, n1, n2 = finalize_slice_size(tuple(mol.space), pixel_size, dz, lateral_size, n_slices)
    b = backend.MultiSlicesBuilder(list(uz), ns, n1, n2, dz, pixel_size[0], pixel_size[1])
    if not add_water and b.atoms_path:
        # same bins and slices without the dense histogram
        return b.build_from_atoms(mol.coordinates, cnt)
    h = b.bin_atoms_multi_slices(mol.coordinates, cnt)
    if add_water:
        h = b.add_water(h)
    return b.make_multi_slices(h)
