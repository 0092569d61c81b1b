"""Imaging pipeline (emsim/pipe.py:9-91) on the GB300 backend.

``Pipe.run`` keeps the reference's semantics - centralize, build the slices with
lateral size ``roi`` and thickness ``slice_thickness`` (optionally with voxel water),
plane wave, multislice, objective lens, |psi|^2 - and forms the image in one fused
engine call after the slices exist.  ``run_batch`` forms many images, one engine call
per group of equal (n_slices, roi).  With ``cuda_graphs=True`` a batch whose structure
(atom and molecule counts, stack shapes, elements, defocus values) was seen before
replays one CUDA graph of its slice builds and image formation instead of launching
them one by one.
"""
from __future__ import annotations

import os
from collections import defaultdict
from typing import List, Optional, Sequence, Tuple, Union

import numpy as np
import torch

from . import _native
from . import atoms as atm
from . import backend, pot, shard, tem, wave


# chunked run_batch: at least this many molecules and atoms per chunk, at most _MAX_CHUNKS
_CHUNK_MIN_MOLS = 64
_CHUNK_MIN_ATOMS = 1 << 21
_MAX_CHUNKS = 2
# a group whose slice stack would exceed this many bytes is imaged with its slices built
# a few pairs at a time (emsim_gb300_image_from_atoms_z), in chunk buffers of about
# _SLICE_CHUNK_BYTES; the images are bitwise the same.  Measured on the 2048^2 x 400-slice
# slab: 16 pairs per chunk (1 GiB) cost 1.3 % against the whole 6.7 GB stack, 1 pair 12 %.
_STACK_LIMIT_BYTES = 2 << 30
_SLICE_CHUNK_BYTES = 1 << 30


def slice_chunk_pairs(n_images: int, n1: int, n2: int) -> int:
    """Slice pairs per chunk of the chunked image formation: the chunk's complex work and
    its two float32 slices take 16 bytes per pixel per pair and image."""
    return max(1, _SLICE_CHUNK_BYTES // (16 * n_images * n1 * n2))


def _fast_len(n: int) -> bool:
    return 8 <= n <= 4096 and (n & (n - 1)) == 0


class _GraphCache:
    """CUDA graphs of a Pipe's batches, per input-buffer set, keyed by batch structure.

    A structure is captured the second time it is seen (the first run creates the plans
    and tables the launches use, which allocates and so cannot be captured), replayed
    from then on.  At most ``max_entries`` graphs are kept per buffer set (least recently
    used dropped); a buffer set that grows drops all of its graphs, whose launches read
    the old buffers."""

    def __init__(self, max_entries: int = 2, max_seen: int = 4096):
        self.max_entries = max_entries
        self.max_seen = max_seen
        self._entries = {}  # buf_key -> OrderedDict(key -> entry)
        self._seen = {}

    def get(self, buf_key, key):
        ent = self._entries.get(buf_key)
        if ent is None or key not in ent:
            return None
        ent.move_to_end(key)
        return ent[key]

    def sighting(self, buf_key, key) -> int:
        """How many times (this one included) the structure was met on this buffer set."""
        if len(self._seen) >= self.max_seen:
            self._seen.clear()
        n = self._seen.get((buf_key, key), 0) + 1
        self._seen[(buf_key, key)] = n
        return n

    def put(self, buf_key, key, entry) -> None:
        from collections import OrderedDict
        ent = self._entries.setdefault(buf_key, OrderedDict())
        ent[key] = entry
        ent.move_to_end(key)
        while len(ent) > self.max_entries:
            ent.popitem(last=False)

    def drop(self, buf_key) -> None:
        self._entries.pop(buf_key, None)
        for k in [k for k in self._seen if k[0] == buf_key]:
            del self._seen[k]

    def __len__(self) -> int:
        return sum(len(v) for v in self._entries.values())


class Pipe:
    def __init__(self, microscope: tem.TEM, resolution: float, slice_thickness: float,
                 roi: Optional[Union[int, Tuple[int, int]]] = None, n_slices: Optional[int] = None,
                 add_water: bool = True, upto_exit_wave: bool = False, cuda_graphs: bool = False):
        self._resolution = resolution
        # run_batch / submit_batch replay a CUDA graph for a batch structure seen before
        self.cuda_graphs = cuda_graphs
        self._graphs = _GraphCache()
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
        """Weak-phase image: one projected slice, transmit, lens, |psi|^2 (pipe.py:57-77)."""
        return backend.intensity(self.lens_propagate(self.get_exit_wave_wpo(mol)))

    def run(self, mol):
        """Image of one molecule, (n1, n2) float32 on the device."""
        if not self.add_water and not self.microscope.partially_coherent:
            return backend._wrap(self.run_batch([mol])[0])
        slices = self.build_slices(mol)
        wp = self._propagator(slices.shape[-2:])
        return self._form_image(wp, slices, self.microscope.defocus)

    def _form_image(self, wp, slices, defocus):
        """plane wave -> multislice -> lens -> |psi|^2 of one (n_slices, n1, n2) stack,
        partially coherent when the microscope says so."""
        m = self.microscope
        if m.partially_coherent:
            return wp.image_partially_coherent(slices, self.slice_thickness, m.electron_dose, m.cs_mm, defocus,
                                               m.aperture, m.focal_spread, m.illumination_angle, m.n_focal)
        return wp.image(slices, self.slice_thickness, m.electron_dose, m.cs_mm, defocus, m.aperture)

    def _geometry(self, mol: atm.AtomList):
        """Centralize, group by element and size the slice stack (pot.py:29-48)."""
        mol = atm.centralize(mol)
        must = [1, 8] if self.add_water else []
        mol, uz, cnt = atm.sort_elements_and_count(mol, must)
        ns, n1, n2 = pot.finalize_slice_size(tuple(mol.space), (self._pixel_size, self._pixel_size),
                                             self.slice_thickness, self.roi, None)
        return mol, uz, cnt, (ns, n1, n2)

    def _stage(self, n_atoms: int):
        """Pinned host staging buffers (grown on demand) for coordinates and Z."""
        if getattr(self, "_pin_xyz", None) is None or self._pin_xyz.shape[0] < n_atoms:
            cap = max(n_atoms, 1024)
            self._pin_xyz = torch.empty((cap, 3), dtype=torch.float32, pin_memory=True)
            self._pin_z = torch.empty(cap, dtype=torch.int32, pin_memory=True)
        return self._pin_xyz[:n_atoms], self._pin_z[:n_atoms]

    def _fill_stage(self, mols, offsets, nx, nz):
        """Copy the molecules' coordinates and Z into the pinned staging buffers; large
        batches are copied by a small thread pool (numpy releases the GIL in the copy and
        cast loops), which keeps the host side of ``run_batch`` short next to the GPU's."""
        def fill(i):
            nx[offsets[i]:offsets[i + 1]] = mols[i].coordinates
            nz[offsets[i]:offsets[i + 1]] = mols[i].elements

        if len(mols) < 4 or int(offsets[-1]) < (1 << 18):
            for i in range(len(mols)):
                fill(i)
            return
        if getattr(self, "_pool", None) is None:
            from concurrent.futures import ThreadPoolExecutor
            self._pool = ThreadPoolExecutor(max_workers=max(1, min(8, (os.cpu_count() or 2) // 2)))
        list(self._pool.map(fill, range(len(mols))))

    def run_batch(self, mols: Sequence[atm.AtomList], defocus: Optional[Sequence[float]] = None,
                  to_host: bool = False, rois: Optional[Sequence] = None) -> List:
        """Images of many molecules (optionally one defocus each), in input order.

        The molecules travel to the device once; centralisation, element sets, binning
        and slice building run there (emsim_gb300_centralize, build_slices_z).  Only the
        per-molecule extents and element masks come back to size the slice stacks.
        Molecules of one lateral size share one slice-build call and one image-formation
        call even when their slice counts differ (a ragged batch: each molecule is binned
        on its own slice axis, and each multislice step runs only over the images that
        still have a slice); each group uses the union of its molecules' elements (an
        absent element adds exactly zero to a slice), and groups of different sizes run on
        their own CUDA streams.  ``to_host``: return numpy images, copied with one
        transfer per group.  ``rois``: a lateral size (int or (n1, n2)) per molecule in
        place of the pipe's roi."""
        if self.add_water or self.microscope.partially_coherent:
            imgs = self._run_batch_host(mols, defocus)
            return [im.get() for im in imgs] if to_host else imgs
        if to_host:
            return self.submit_batch(mols, defocus, rois).result()
        done = self._queue_batch(mols, defocus, rois, torch.cuda.current_stream(), "sync")
        out: List = [None] * len(mols)
        for idx, imgs in done:
            for j, i in enumerate(idx):
                out[i] = imgs[j]
        return out

    def submit_batch(self, mols: Sequence[atm.AtomList], defocus: Optional[Sequence[float]] = None,
                     rois: Optional[Sequence] = None) -> "PendingImages":
        """Queue the images of many molecules and their copy to page-locked host memory,
        and return without waiting for the GPU.  ``result()`` of the returned object gives
        what ``run_batch(..., to_host=True)`` gives.

        Successive batches alternate between two sets of CUDA streams, so the host side of
        the next batch (staging its atoms, the H2D copy, the front-end's small sync that
        sizes the stacks, the launches) runs while the GPU forms this batch's images::

            pending = p.submit_batch(batch0)
            for nxt in batches[1:]:
                following = p.submit_batch(nxt)
                consume(pending.result())
                pending = following
            consume(pending.result())
        """
        if self.add_water or self.microscope.partially_coherent:
            return PendingImages.completed([im.get() for im in self._run_batch_host(mols, defocus)])
        slot = getattr(self, "_slot", 1) ^ 1
        self._slot = slot
        base = self._chunk_stream((slot, "base"))
        base.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(base):
            done = self._queue_batch(mols, defocus, rois, base, slot)
            groups = []
            for idx, imgs in done:
                # one transfer per group into page-locked memory from torch's caching host
                # allocator (a pageable copy of 33 MB takes ~2.4 ms against ~0.2 ms)
                h = torch.empty(imgs.shape, dtype=imgs.dtype, pin_memory=True)
                h.copy_(imgs, non_blocking=True)
                groups.append((idx, h, imgs))
            ev = torch.cuda.Event()
            ev.record(base)
        return PendingImages(len(mols), groups, ev)

    def shard_costs(self, mols: Sequence[atm.AtomList], rois: Optional[Sequence] = None) -> List[float]:
        """Estimated cost of each molecule's image - slices x pixels x log2(pixels), the FFT
        work of its multislice loop - from the host coordinates' extent, which sizes its
        stack exactly as the device front-end will (pot.finalize_slice_size)."""
        costs = []
        for i, mol in enumerate(mols):
            lateral = self.roi if rois is None else (
                (rois[i], rois[i]) if isinstance(rois[i], (int, np.integer)) else tuple(rois[i]))
            ns, n1, n2 = pot.finalize_slice_size(tuple(mol.space), (self._pixel_size, self._pixel_size),
                                                 self.slice_thickness, lateral, None)
            costs.append(shard.image_cost(ns, n1, n2))
        return costs

    def run_sharded(self, mols: Sequence[atm.AtomList], defocus: Optional[Sequence[float]] = None,
                    rois: Optional[Sequence] = None, group=None) -> Optional[List[np.ndarray]]:
        """Images of many molecules over the ranks of a torch.distributed group, one GPU per
        rank (emsim/simulator.py:64-91 spreads its work over threads of one process; here
        over processes).  Every rank passes the same molecules; each images the share that
        the deterministic cost partition (shard.partition: longest first, to the least
        loaded rank) gives it with ``run_batch`` on its current device, and the host images
        are gathered to rank 0 (torch.distributed.gather_object) - no collective touches the
        device data.  Rank 0 returns the images in input order, the other ranks None."""
        import torch.distributed as dist
        rank, world = dist.get_rank(group), dist.get_world_size(group)
        mine = shard.my_share(self.shard_costs(mols, rois), rank, world)
        local = {}
        if mine:
            imgs = self.run_batch([mols[i] for i in mine], None if defocus is None else [defocus[i] for i in mine],
                                  to_host=True, rois=None if rois is None else [rois[i] for i in mine])
            local = {i: img for i, img in zip(mine, imgs)}
        return shard.gather_to_root(local, len(mols), rank, world, group)

    def _queue_batch(self, mols, defocus, rois, main, slot) -> List:
        """Queue a batch's device work so that it completes in stream ``main``; returns
        [(indices, images)] with images (len(indices), n1, n2) on the device."""
        sizes = [len(mol.elements) for mol in mols]
        if any(s == 0 for s in sizes):
            raise ValueError("zero-size array to reduction operation minimum which has no identity")
        nm = len(mols)
        # Large batches (128 molecules and 4 M atoms and more) run in two chunks, each on its
        # own stream: while the GPU builds and images the first, the host stages the second
        # and its front-end (H2D, centralisation, the sync that sizes the stacks) runs beside
        # it.  Images are independent, so the results do not depend on the chunking.
        n_chunks = 1
        if nm >= 2 * _CHUNK_MIN_MOLS and sum(sizes) >= 2 * _CHUNK_MIN_ATOMS:
            n_chunks = int(min(_MAX_CHUNKS, nm // _CHUNK_MIN_MOLS, sum(sizes) // _CHUNK_MIN_ATOMS))
        bounds = np.linspace(0, nm, n_chunks + 1).round().astype(int)
        done = []
        streams = []
        for c in range(n_chunks):
            a, b = int(bounds[c]), int(bounds[c + 1])
            st = main if n_chunks == 1 else self._chunk_stream((slot, c))
            if st is not main:
                st.wait_stream(main)
                streams.append(st)
            with torch.cuda.stream(st):
                part = self._launch_chunk(mols[a:b], None if defocus is None else defocus[a:b],
                                          None if rois is None else rois[a:b], (slot, c))
                for idx, imgs in part:
                    if st is not main:
                        imgs.record_stream(main)
                    done.append(([a + i for i in idx], imgs))
        for st in streams:
            main.wait_stream(st)
        return done

    def _chunk_stream(self, key):
        pool = getattr(self, "_streams", None)
        if pool is None:
            pool = self._streams = {}
        dev = torch.cuda.current_device()
        if (dev, key) not in pool:
            pool[(dev, key)] = torch.cuda.Stream()
        return pool[(dev, key)]

    def _inputs(self, buf_key, n_atoms: int, nm: int):
        """Device input buffers of one buffer set (grown on demand), so that a replayed
        graph finds the batch at the addresses it was captured with."""
        bufs = getattr(self, "_in_bufs", None)
        if bufs is None:
            bufs = self._in_bufs = {}
        dev = backend._device()
        b = bufs.get(buf_key)
        if b is None or b["xyz"].device != dev or b["xyz"].shape[0] < n_atoms or b["shift"].shape[0] < nm:
            if b is not None and b["busy"] is not None:
                # the old buffers and the graphs that read them go: their last batch must be done
                b["busy"].synchronize()
            cap = max(n_atoms, 1024 if b is None else b["xyz"].shape[0])
            capm = max(nm, 16 if b is None else b["shift"].shape[0])
            b = {"xyz": torch.empty((cap, 3), dtype=torch.float32, device=dev),
                 "z": torch.empty(cap, dtype=torch.int32, device=dev),
                 "off": torch.empty(capm + 1, dtype=torch.int32, device=dev),
                 "shift": torch.empty((capm, 3), dtype=torch.float32, device=dev),
                 "space": torch.empty((capm, 3), dtype=torch.float32, device=dev),
                 "present": torch.empty((capm, 4), dtype=torch.int32, device=dev),
                 "busy": None}
            bufs[buf_key] = b
            self._graphs.drop(buf_key)
        return b

    def _group_work(self, key, idx, ss, uz, dfs, xyz, zz, off, shift, nm):
        """The device work of one group (slices and images) as prepared launches, and
        whether it can be captured (the atoms path; the host-side slice build is not)."""
        m = self.microscope
        n1, n2 = key[-2:]
        b = backend.MultiSlicesBuilder(uz, ss[0], n1, n2, self.slice_thickness, self._pixel_size, self._pixel_size)
        wp = self._propagator((n1, n2))
        ragged = ss[0] != ss[-1]
        if not b.atoms_path:
            def host_work():
                stack = torch.stack([self.build_slices(self._mols_now[i]) for i in idx])
                return wp.image(stack, self.slice_thickness, m.electron_dose, m.cs_mm, dfs, m.aperture,
                                n_batch=len(idx))
            return [host_work], False
        # too large a stack to hold: slices built a few pairs at a time
        if not ragged and 4 * len(idx) * ss[0] * n1 * n2 > _STACK_LIMIT_BYTES:
            return [backend.prepare_image_from_device_atoms(
                b, wp, xyz, zz, off, shift, idx, nm, m.electron_dose, m.cs_mm, dfs, m.aperture,
                slice_chunk_pairs(len(idx), n1, n2))], True
        build = backend.prepare_build_slices_from_device_atoms(b, xyz, zz, off, shift, idx, nm,
                                                               slot_slices=ss if ragged else None)
        if ragged:
            image = backend.prepare_image_ragged(wp, build.result, ss, self.slice_thickness, m.electron_dose, m.cs_mm,
                                                 dfs, m.aperture)
        else:
            image = wp.prepare_image(build.result, self.slice_thickness, m.electron_dose, m.cs_mm, dfs, m.aperture,
                                     n_batch=len(idx))
        return [build, image], True

    def _launch_chunk(self, mols, defocus, rois, buf_key=None):
        """Queue the device work of one chunk on the current stream (groups of other
        lateral sizes on side streams joined back into it); returns [(indices, images)]."""
        m = self.microscope
        dev = backend._device()
        nm = len(mols)
        sizes = [len(mol.elements) for mol in mols]
        offsets = np.zeros(nm + 1, dtype=np.int64)
        offsets[1:] = np.cumsum(sizes)
        n_atoms = int(offsets[-1])
        hx, hz = self._stage(n_atoms)
        self._fill_stage(mols, offsets, hx.numpy(), hz.numpy())
        graphs = self.cuda_graphs and buf_key is not None
        main = torch.cuda.current_stream()
        off_h = torch.from_numpy(offsets.astype(np.uint32).view(np.int32))
        if graphs:
            bufs = self._inputs(buf_key, n_atoms, nm)
            if bufs["busy"] is not None:
                main.wait_event(bufs["busy"])  # the last batch on these buffers is done with them
            xyz, zz = bufs["xyz"][:n_atoms], bufs["z"][:n_atoms]
            off, shift = bufs["off"][:nm + 1], bufs["shift"][:nm]
            space, present = bufs["space"][:nm], bufs["present"][:nm]
            xyz.copy_(hx, non_blocking=True)
            zz.copy_(hz, non_blocking=True)
            off.copy_(off_h)
        else:
            xyz = hx.to(dev, non_blocking=True)
            zz = hz.to(dev, non_blocking=True)
            off = off_h.to(dev)
            shift = torch.empty((nm, 3), dtype=torch.float32, device=dev)
            space = torch.empty((nm, 3), dtype=torch.float32, device=dev)
            present = torch.empty((nm, 4), dtype=torch.int32, device=dev)
        P = backend._ptr
        backend._native.call("emsim_gb300_centralize", P(xyz), P(zz), P(off), nm, P(shift), P(space), P(present),
                             backend._stream())
        space_h = space.cpu().numpy()
        mask_h = present.cpu().numpy().view(np.uint32)
        # one group per lateral size on the fused path (a ragged batch: every molecule keeps
        # its own slice count), one per full stack shape otherwise
        groups = defaultdict(list)
        n_sl = {}
        for i in range(nm):
            lateral = self.roi if rois is None else (
                (rois[i], rois[i]) if isinstance(rois[i], (int, np.integer)) else tuple(rois[i]))
            ns, n1, n2 = pot.finalize_slice_size(tuple(space_h[i]), (self._pixel_size, self._pixel_size),
                                                 self.slice_thickness, lateral, None)
            n_sl[i] = ns
            fast = _fast_len(n1) and _fast_len(n2)
            groups[(n1, n2) if fast else (ns, n1, n2)].append(i)
        plan = []
        for key, idx in groups.items():
            idx = sorted(idx, key=lambda i: -n_sl[i])  # longest stack first
            ss = [n_sl[i] for i in idx]
            union = np.bitwise_or.reduce(mask_h[idx], axis=0)
            uz = [32 * w + b for w in range(4) for b in range(32) if (int(union[w]) >> b) & 1]
            dfs = [float(m.defocus if defocus is None else defocus[i]) for i in idx]
            plan.append((key, idx, ss, uz, dfs))
        self._mols_now = mols  # read by the host-side slice build of groups off the atoms path
        try:
            if graphs:
                done = self._graph_chunk(buf_key, plan, n_atoms, nm, xyz, zz, off, shift, main)
                if done is not None:
                    ev = torch.cuda.Event()
                    ev.record(main)
                    bufs["busy"] = ev
                    return done
            ready = torch.cuda.Event()
            ready.record(main)
            side, done = [], []
            for key, idx, ss, uz, dfs in plan:
                # lateral sizes overlap on the GPU: each group runs on its own stream
                st = torch.cuda.Stream() if len(plan) > 1 else main
                st.wait_event(ready)
                with torch.cuda.stream(st):
                    work, _ = self._group_work(key, idx, ss, uz, dfs, xyz, zz, off, shift, nm)
                    for w in work:
                        imgs = w()
                    imgs = backend._wrap(imgs.reshape(len(idx), *key[-2:]))
                    if st is not main:
                        imgs.record_stream(main)
                if st is not main:
                    side.append(st)
                done.append((idx, imgs))
            for st in side:
                main.wait_stream(st)
            if graphs:
                ev = torch.cuda.Event()
                ev.record(main)
                bufs["busy"] = ev
            return done
        finally:
            self._mols_now = None

    def _graph_chunk(self, buf_key, plan, n_atoms, nm, xyz, zz, off, shift, main):
        """The chunk's groups through a CUDA graph: replayed if this structure was
        captured, captured on its second sighting, else None (run it eagerly).  Images
        come back as copies, so that the next replay does not overwrite them."""
        m = self.microscope
        key = (n_atoms, nm, tuple((k, tuple(idx), tuple(ss), tuple(uz), tuple(dfs)) for k, idx, ss, uz, dfs in plan),
               (float(m.electron_dose), float(m.cs_mm), float(m.aperture), float(m.wave_length)),
               float(self.slice_thickness), float(self._pixel_size), backend.get_precision())
        ent = self._graphs.get(buf_key, key)
        if ent is None:
            if self._graphs.sighting(buf_key, key) < 2:
                return None
            work = []
            for k, idx, ss, uz, dfs in plan:
                w, ok = self._group_work(k, idx, ss, uz, dfs, xyz, zz, off, shift, nm)
                if not ok:
                    return None
                work.append((k, idx, w))
            cap = self._chunk_stream((buf_key, "capture"))
            cap.wait_stream(main)
            g = torch.cuda.CUDAGraph()
            # entering the capture synchronises the device, so the graph that put() may drop
            # below (least recently used) has no replay in flight
            with torch.cuda.graph(g, stream=cap):
                for _, _, w in work:
                    for step in w:
                        step()
            main.wait_stream(cap)
            ent = {"graph": g, "work": work}
            self._graphs.put(buf_key, key, ent)
        ent["graph"].replay()
        return [(idx, backend._wrap(w[-1].result.reshape(len(idx), *k[-2:]).clone())) for k, idx, w in ent["work"]]

    def _run_batch_host(self, mols, defocus=None) -> List:
        """run_batch with the front-end on the host (voxel water needs the histograms) or
        one image at a time (partial coherence)."""
        m = self.microscope
        if m.partially_coherent:
            out = []
            for i, mol in enumerate(mols):
                s = self.build_slices(mol)
                wp = self._propagator(s.shape[-2:])
                out.append(self._form_image(wp, s, m.defocus if defocus is None else defocus[i]))
            return out
        out: List = [None] * len(mols)
        groups = defaultdict(list)
        built = {}
        for i, mol in enumerate(mols):
            s = self.build_slices(mol)
            built[i] = s
            groups[tuple(s.shape)].append(i)
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


class PendingImages:
    """Images of a batch queued by ``Pipe.submit_batch``: the device work and the copy to
    page-locked host memory are in flight.  ``result()`` waits for them and returns the
    numpy images in input order (each array keeps its page-locked buffer alive)."""

    def __init__(self, n: int, groups, event):
        self._n = n
        self._groups = groups  # [(indices, page-locked host tensor, device tensor)]
        self._event = event
        self._out = None

    @classmethod
    def completed(cls, images: List) -> "PendingImages":
        p = cls(len(images), None, None)
        p._out = list(images)
        return p

    def done(self) -> bool:
        """True once result() will not wait."""
        return self._out is not None or self._event.query()

    def result(self) -> List[np.ndarray]:
        """The images; raises ``DeviceWaitTimeout`` when a kernel gave up a bounded wait."""
        if self._out is None:
            self._event.synchronize()
            _native.raise_on_device_error()
            out: List = [None] * self._n
            for idx, h, _ in self._groups:
                a = h.numpy()
                for j, i in enumerate(idx):
                    out[i] = a[j]
            self._out = out
            self._groups = None
        return self._out
