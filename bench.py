"""Throughput benchmark of the emsim multislice hot path on GB300.

Headline workload: the amorphous-carbon slab, 838,861 C atoms uniform at 0.1 A^-3 over
204.8 x 204.8 x 200 A (seeded), imaged on a 2048 x 2048 wave at pixel 0.1 A through 400
slices of 0.5 A, 300 keV, Cs 1.0 mm, Scherzer defocus and aperture, plain FP32: atom
binning -> projected-potential slices -> multislice -> lens -> |psi|^2.  One step images
eight such slabs (eight seeds, --batch).  ``value`` times that step with its atoms
resident in HBM (L2 flushed by a 256 MiB write before every step, CUDA events on the
launching stream); ``e2e`` runs the same images through the public ``Pipe.submit_batch``
API from host atoms to host images, every step copying the atoms in and the images out.

Extras beside the headline (outside its timed region): slice-steps/s at 256^2, 512^2
and 2048^2 against the HBM roofline; the 512^2 x 64-slice x 32-defocus forward of the
differentiation workload; the 50k-atom blob at 256^2 (128 images per step); the mixed
batch; the split-BF16 passes; the reference's cuFFT design on the same slices; forward
+ backward of the differentiation workload.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU (torchrun): every rank images its own slab (weak scaling, no collective on the
data path); rank 0 prints the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# amorphous-carbon slab (the headline)
SLAB = dict(n=2048, pixel=0.1, n_slices=400, dz=0.5, kev=300.0, cs_mm=1.0, dose=20.0, lateral=204.8,
            thickness=200.0, density=0.1)
# 50k-atom C/N/O/S blob at 256^2 (extra)
BLOB = dict(n_atoms=50_000, radius=40.0, roi=256, resolution=2.0, slice_thickness=2.0, kev=200.0,
            cs_mm=1.3, defocus=700.0, aperture=10e-3, dose=20.0)
# differentiation geometry, forward only (extra)
DIFF = dict(n_atoms=20_000, radius=50.0, n=512, pixel=0.5, n_slices=64, dz=1.0, kev=200.0, cs_mm=1.3,
            aperture=10e-3, dose=20.0, n_defocus=32)

METRIC = "images/s"
WORKLOAD = ("amorphous-carbon slab: 838,861 C atoms uniform at 0.1 A^-3 over 204.8 x 204.8 x 200 A, "
            "2048^2 wave at pixel 0.1 A, 400 slices of 0.5 A, 300 keV, Cs 1.0 mm, Scherzer defocus and "
            "aperture, plain FP32")
CONFIG = {"workload": WORKLOAD, "image": "2048x2048", "slices": 400}


def slab_atoms(seed: int):
    from emsim_gb300.synth import carbon_slab  # seeded synthetic input generator
    return carbon_slab(seed, SLAB["lateral"], SLAB["thickness"], SLAB["density"])


def scherzer():
    from emsim_gb300 import physics
    lam = physics.electron_wave_length_angstrom(SLAB["kev"])
    return physics.scherzer_condition(lam, SLAB["cs_mm"])


def rank_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


# ---------------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------------
class ClockSampler:
    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.rows = []

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        sm = [float(r[1]) for r in self.rows if len(r) > 2 and r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if len(r) > 2 and r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows if len(r) >= 9 for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def timed(torch, fn, reps: int, flush=None, warm: int = 1):
    """Median seconds of fn() over reps calls, CUDA events on the current stream, L2
    flushed before each call when ``flush`` (a device buffer larger than L2) is given."""
    for _ in range(warm):
        fn()
    ts = []
    for _ in range(reps):
        if flush is not None:
            flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        fn()
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    return float(np.median(ts))


def scan_launches(n: int) -> int:
    """Kernel launches of the engine's exclusive scan over n words (chunks of 4096)."""
    return 2 + (1 if n > 4096 else 0)


def build_launches(n_img: int, n_elems: int, n_pairs: int, n1: int) -> int:
    """Kernel launches of emsim_gb300_build_slices: group scan, bucket, bucket scan,
    scatter, column pass, inverse row pass."""
    return scan_launches(n_img * n_elems) + 1 + scan_launches(n_img * n_elems * n_pairs * n1) + 1 + 2


# ---------------------------------------------------------------------------------
# device-resident steps
# ---------------------------------------------------------------------------------
class DeviceImages:
    """Device-resident atoms and buffers of B molecules that share one element set and
    one slice count; run() queues one full step: slices of all molecules straight from
    their atoms (emsim_gb300_build_slices), then plane wave -> multislice -> lens ->
    |psi|^2 (emsim_gb300_multislice_image)."""

    def __init__(self, torch, mols, pixel, dz, lateral, kev, dose, cs_mm, defocus, aperture):
        from emsim_gb300 import atoms, backend, pot
        self.torch, self.backend = torch, backend
        dev = torch.device("cuda", torch.cuda.current_device())
        geo = []
        for el, xyz in mols:
            mol = atoms.centralize(atoms.AtomList(el, xyz))
            mol, uz, cnt = atoms.sort_elements_and_count(mol)
            ns, n1, n2 = pot.finalize_slice_size(tuple(mol.space), (pixel, pixel), dz, lateral, None)
            geo.append((mol.coordinates, tuple(int(z) for z in uz), cnt, ns, n1, n2))
        keys = {(g[1], g[3], g[4], g[5]) for g in geo}
        if len(keys) != 1:
            raise RuntimeError(f"molecules of one step need equal elements and stack shapes, got {sorted(keys)}")
        (uz, ns, n1, n2), = keys
        self.uz, self.ns, self.n1, self.n2, self.B = uz, ns, n1, n2, len(mols)
        self.dz, self.dose, self.cs_mm, self.aperture = dz, dose, cs_mm, aperture
        self.pixel, self.kev = pixel, kev
        self.builder = backend.MultiSlicesBuilder(list(uz), ns, n1, n2, dz, pixel, pixel)
        xyz = np.ascontiguousarray(np.concatenate([g[0] for g in geo]))
        counts = np.stack([g[2] for g in geo]).astype(np.uint32)
        self.n_atoms = int(xyz.shape[0])
        self.coords = torch.from_numpy(xyz).to(dev)
        self.counts = torch.from_numpy(counts.view(np.int32)).to(dev)
        self.slices = torch.empty((self.B, ns, n1, n2), dtype=torch.float32, device=dev)
        self.work = torch.empty((self.B, n1, n2), dtype=torch.complex64, device=dev)
        self.img = torch.empty((self.B, n1, n2), dtype=torch.float32, device=dev)
        lib = backend._native.load()
        self.ws_bytes = int(lib.emsim_gb300_build_slices_workspace_size(self.builder._plan.handle, self.n_atoms,
                                                                       self.B))
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=dev)
        self.wp = backend.WavePropagator(n1, n2, pixel, pixel, kev)
        self.df = np.full(self.B, defocus, dtype=np.float64)

    def launches_per_step(self) -> int:
        n_pairs = (self.ns + 1) // 2
        lens = math.ceil(self.B / 64)
        return build_launches(self.B, len(self.uz), n_pairs, self.n1) + 2 * self.ns + lens + 1

    def run_build(self):
        P = self.backend._ptr
        st = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        self.backend._native.call("emsim_gb300_build_slices", self.builder._plan.handle, P(self.coords),
                                  self.n_atoms, P(self.counts), self.B, P(self.slices), P(self.ws), self.ws_bytes, st)

    def run_image(self):
        """plane wave -> multislice -> lens -> |psi|^2 of all molecules from the built slices."""
        P = self.backend._ptr
        st = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        self.backend._native.call(
            "emsim_gb300_multislice_image", self.wp._plan.handle, P(self.slices), self.ns,
            self.ns * self.n1 * self.n2, self.dz, self.dose, self.cs_mm,
            self.df.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), self.B, self.aperture, P(self.img),
            P(self.work), None, self.B, st)

    def run(self):
        self.run_build()
        self.run_image()

    def graph(self):
        """The step captured once in a CUDA graph (after warm-up)."""
        torch = self.torch
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=s):
                self.run()
        torch.cuda.current_stream().wait_stream(s)
        g.replay()
        torch.cuda.synchronize()
        return g


def slab_step(torch, seeds) -> DeviceImages:
    """The headline step: one image of each seeded slab in ``seeds``."""
    df, ap = scherzer()
    return DeviceImages(torch, [slab_atoms(s) for s in seeds], SLAB["pixel"], SLAB["dz"], SLAB["n"], SLAB["kev"],
                        SLAB["dose"], SLAB["cs_mm"], df, ap)


def chunked_extra(torch, seed: int, flush, reps: int = 3) -> dict:
    """The headline image through emsim_gb300_image_from_atoms_z (slices built a few pairs
    at a time, never the whole 6.7 GB stack) at 1 and 16 slice pairs per chunk, with the
    device memory each needs; the images are bitwise those of the headline step."""
    from emsim_gb300 import backend, pot
    el, xyz = slab_atoms(seed)
    dev = torch.device("cuda", torch.cuda.current_device())
    xyz_d = torch.from_numpy(xyz).to(dev)
    z_d = torch.from_numpy(el.astype(np.int32)).to(dev)
    off = torch.tensor([0, len(el)], dtype=torch.int32, device=dev)
    shift = torch.empty((1, 3), dtype=torch.float32, device=dev)
    space = torch.empty((1, 3), dtype=torch.float32, device=dev)
    P = backend._ptr
    backend._native.call("emsim_gb300_centralize", P(xyz_d), P(z_d), P(off), 1, P(shift), P(space), None,
                         backend._stream())
    n, d, dz = SLAB["n"], SLAB["pixel"], SLAB["dz"]
    ns, _, _ = pot.finalize_slice_size(tuple(space.cpu().numpy()[0]), (d, d), dz, n, None)
    b = backend.MultiSlicesBuilder([6], ns, n, n, dz, d, d)
    wp = backend.WavePropagator(n, n, d, d, SLAB["kev"])
    df, ap = scherzer()
    lib = backend._native.load()
    out = {"workload": "the headline image, slices built chunk by chunk (emsim_gb300_image_from_atoms_z)",
           "whole_stack_bytes": 4 * ns * n * n}
    for chunk in (1, 16):
        t = timed(torch, lambda: backend.image_from_device_atoms(b, wp, xyz_d, z_d, off, shift, [0], 1, SLAB["dose"],
                                                                 SLAB["cs_mm"], [df], ap, chunk), reps, flush)
        out[f"pairs_{chunk}"] = {"images_per_s": round(1.0 / t, 3), "workspace_bytes": int(
            lib.emsim_gb300_image_from_atoms_workspace_size(b._plan.handle, len(el), 1, chunk))}
    return out


def slice_step_on(torch, db: DeviceImages, peak_gbs: float, reps: int = 3, flush=None) -> dict:
    """Average duration of one slice step (fused row pass + column pass) of the step's
    own waves and slices: CUDA events around multislice_propagate through all slices of
    all images, divided by the number of steps (+1/2 for the closing inverse row pass)."""
    w = torch.empty((db.B, db.n1, db.n2), dtype=torch.complex64, device=db.slices.device)
    w.fill_(1.0)
    t = timed(torch, lambda: db.wp.multislice_propagate(w, db.slices, db.dz), reps, flush)
    per_step = t / (db.ns + 0.5)
    algo = 20.0 * db.n1 * db.n2 * db.B  # psi read 8 + psi write 8 + V read 4 per pixel
    return {"n": db.n1, "images": db.B, "slices": db.ns, "step_s": per_step, "slice_steps_per_s": db.B / per_step,
            "achieved_gbs": algo / per_step / 1e9, "frac": algo / per_step / 1e9 / peak_gbs,
            "algorithmic_bytes": algo}


def slice_step_roofline(torch, backend, n: int, n_img: int, n_slices: int, peak_gbs: float, reps: int = 5):
    """Slice-step duration on a batch of n_img waves of n x n through n_slices random
    slices (multislice_propagate, CUDA events, L2 flushed)."""
    dev = torch.device("cuda", torch.cuda.current_device())
    wp = backend.WavePropagator(n, n, 0.5, 0.5, 200.0)
    w = torch.ones((n_img, n, n), dtype=torch.complex64, device=dev)
    sl = torch.rand((n_img, n_slices, n, n), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    t = timed(torch, lambda: wp.multislice_propagate(w, sl, 2.0), reps, flush, warm=2)
    per_step = t / (n_slices + 0.5)
    algo = 20.0 * n * n * n_img
    return {"n": n, "images": n_img, "slices": n_slices, "step_s": per_step,
            "slice_steps_per_s": n_img / per_step, "achieved_gbs": algo / per_step / 1e9,
            "frac": algo / per_step / 1e9 / peak_gbs}


def build_roofline(torch, db: DeviceImages, peak_gbs: float, reps: int = 3, flush=None) -> dict:
    """The histogram-free slice build of a step (emsim_gb300_build_slices) timed alone
    against its algorithmic bytes: 16 B per atom read (float32 xyz + the element counts'
    share) and 4 B per slice pixel written."""
    t = timed(torch, db.run_build, reps, flush)
    algo = 16.0 * db.n_atoms + 4.0 * db.B * db.ns * db.n1 * db.n2
    return {"kernel": "slice build = bucketing + slice_cols_atoms_kernel + slice_rows_inv_kernel "
                      "(%d image(s), %d slices of %d^2)" % (db.B, db.ns, db.n1),
            "seconds": t, "achieved_gbs": algo / t / 1e9, "frac": algo / t / 1e9 / peak_gbs,
            "algorithmic_bytes": algo}


# ---------------------------------------------------------------------------------
# extras
# ---------------------------------------------------------------------------------
def blob_extra(torch, flush, steps: int, peak: float) -> tuple:
    """The 50k-atom blob workload (roi 256, pixel 1 A, 40 slices of 2 A) with 128 blobs per
    step in a CUDA graph, and the same images through Pipe.submit_batch from host atoms.
    Returns (dict, DeviceImages)."""
    from emsim_gb300 import atoms, pipe, tem
    from emsim_gb300.synth import protein_blob
    W = BLOB
    seeds = list(range(128))
    blobs = [protein_blob(W["n_atoms"], W["radius"], s) for s in seeds]
    db = DeviceImages(torch, blobs, 0.5 * W["resolution"], W["slice_thickness"], W["roi"], W["kev"], W["dose"],
                      W["cs_mm"], W["defocus"], W["aperture"])
    for _ in range(3):
        db.run()
    g = db.graph()
    t = timed(torch, g.replay, steps, flush)
    t_ = tem.TEM(electron_dose=W["dose"], beam_energy_kev=W["kev"], cs_mm=W["cs_mm"], defocus=W["defocus"],
                 aperture=W["aperture"])
    p = pipe.Pipe(t_, resolution=W["resolution"], slice_thickness=W["slice_thickness"], roi=W["roi"],
                  add_water=False)
    mols = [atoms.AtomList(el, xyz) for el, xyz in blobs]
    e2e = pipelined_e2e(torch, p, mols, max(3, min(steps, 6)))
    rl = slice_step_on(torch, db, peak, flush=flush)
    return {"workload": "blob 50k C/N/O/S atoms r=40A, roi 256, pixel 1A, dz 2A, %d slices, 200 keV, Cs 1.3 mm, "
                        "df 700 A, aperture 10 mrad" % db.ns,
            "images_per_step": db.B, "images_per_s": round(db.B / t, 1), "ms_per_step": round(1e3 * t, 4),
            "slice_steps_per_s": round(db.B * db.ns / t, 1), "cuda_graph": True,
            "e2e_images_per_s": round(e2e["value"], 1),
            "slice_step_hbm_frac": round(rl["frac"], 4)}, db


def pipelined_e2e(torch, p, mols, n_steps: int) -> dict:
    """Images/s through Pipe.submit_batch with two batches in flight: the next batch's
    host side (staging, H2D, device front-end, launches) overlaps this batch's device work;
    every step still copies its atoms in and its images out."""
    def run():
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pending = p.submit_batch(mols)
        for _ in range(n_steps - 1):
            following = p.submit_batch(mols)
            host = pending.result()
            pending = following
        host = pending.result()
        torch.cuda.synchronize()
        return len(mols) * n_steps / (time.perf_counter() - t0), host

    run()
    v, host = run()
    return {"value": v, "host": host}


def diff512_forward_extra(torch, flush, reps: int = 5) -> dict:
    """Forward images/s of the differentiation geometry: 20,000 C/N/O/S atoms in a 50 A
    ball, 512^2 at 0.5 A, 64 slices of 1 A (explicit count), 32 defocus values in
    300-1500 A sharing one slice stack: build_from_atoms + WavePropagator.image."""
    from emsim_gb300 import atoms, backend, synth
    W = DIFF
    el, xyz = synth.protein_blob(W["n_atoms"], W["radius"], 77)
    mol, uz, cnt = atoms.sort_elements_and_count(atoms.AtomList(el, xyz))
    dfs = list(np.random.default_rng(78).uniform(300.0, 1500.0, size=W["n_defocus"]))
    b = backend.MultiSlicesBuilder(list(uz), W["n_slices"], W["n"], W["n"], W["dz"], W["pixel"], W["pixel"])
    wp = backend.WavePropagator(W["n"], W["n"], W["pixel"], W["pixel"], W["kev"])
    c = torch.tensor(mol.coordinates, device="cuda")

    def fwd():
        s = b.build_from_atoms(c, cnt)
        return wp.image(s, W["dz"], W["dose"], W["cs_mm"], dfs, W["aperture"])

    t = timed(torch, fwd, reps, flush, warm=2)
    return {"workload": "20k C/N/O/S atoms r=50A, 512^2 at 0.5A, 64 slices of 1A, 32 defocus 300-1500A sharing "
                        "one slice stack, 200 keV; slice build + 32 images (forward only)",
            "images_per_s": round(W["n_defocus"] / t, 1), "ms": round(1e3 * t, 3),
            "slice_steps_per_s": round(W["n_defocus"] * W["n_slices"] / t, 1)}


def differentiation_extra(torch, reps: int = 3) -> dict:
    """Forward + backward of the differentiation workload: 20,000 C/N/O/S atoms in a 50 A
    ball, 512 x 512 at 0.5 A, 64 slices of 1 A, 32 defocus values, MSE against the image
    of a copy jittered by 0.2 A; gradients with respect to the atom coordinates (off-grid
    slices) and the slices (adjoint multislice, sqrt(N) checkpoints)."""
    from emsim_gb300 import atoms, autograd, backend, synth
    el, xyz0 = synth.protein_blob(20_000, 50.0, 77)
    mol, uz, cnt = atoms.sort_elements_and_count(atoms.AtomList(el, xyz0))
    rng = np.random.default_rng(78)
    xyz = mol.coordinates
    jit = (xyz + rng.normal(scale=0.2, size=xyz.shape)).astype(np.float32)
    dfs = list(rng.uniform(300.0, 1500.0, size=32))
    b = backend.MultiSlicesBuilder(list(uz), 64, 512, 512, 1.0, 0.5, 0.5)
    wp = backend.WavePropagator(512, 512, 0.5, 0.5, 200.0)
    with torch.no_grad():
        target = autograd.image(wp, autograd.smooth_slices(b, torch.tensor(jit, device="cuda"), cnt), 1.0, 20.0, 1.3,
                                dfs, 10e-3)
    c = torch.tensor(xyz, device="cuda", requires_grad=True)
    tf, tb = [], []
    for it in range(reps + 2):
        e0, e1, e2 = (torch.cuda.Event(enable_timing=True) for _ in range(3))
        e0.record()
        img = autograd.image(wp, autograd.smooth_slices(b, c, cnt), 1.0, 20.0, 1.3, dfs, 10e-3)
        loss = torch.mean((img - target) ** 2)
        e1.record()
        loss.backward()
        e2.record()
        e2.synchronize()
        c.grad = None
        if it >= 2:
            tf.append(e0.elapsed_time(e1))
            tb.append(e1.elapsed_time(e2))
    f, bw = float(np.median(tf)), float(np.median(tb))
    return {"workload": "20k C/N/O/S atoms r=50A, 512^2 at 0.5A, 64 slices of 1A, 32 defocus 300-1500A, 200 keV, "
                        "MSE vs 0.2A-jittered copy; dLoss/dxyz and dLoss/dV",
            "images_per_s": round(32 / ((f + bw) * 1e-3), 1), "forward_ms": round(f, 3), "backward_ms": round(bw, 3),
            "checkpoint_every": autograd.default_every(64)}


def precision_extra(torch, db: DeviceImages, backend, flush, reps: int = 5):
    """The blob step (eager launches, L2 flushed) with the multislice passes in FP32 and in
    split-BF16 on the tensor cores; returns the timing dict and the split-BF16 image of the
    first blob (its accuracy against FP64 is computed in the CPU leg)."""
    out, img = {}, None
    try:
        for mode in ("fp32", "bf16x3"):
            backend.set_precision(mode)
            t = timed(torch, db.run, reps, flush, warm=2)
            out[mode] = {"images_per_s": round(db.B / t, 1)}
            if mode == "bf16x3":
                img = db.img[0].cpu().numpy()
    finally:
        backend.set_precision("fp32")
    out["workload"] = "the blob step (128 blobs at 256^2), eager launches, L2 flushed before every step"
    out["bf16x3_passes"] = ("256-point row pass (IFFT, transmit, FFT) and column pass (FFT, propagate, IFFT) as "
                            "16x16 four-step DFTs on tcgen05, bf16 hi+lo operands, fp32 accumulation")
    return out, img


def plain_cufft_extra(torch, db: DeviceImages, flush, reps: int = 3) -> dict:
    """The reference's CUDA design on the same GPU and the same slices, as a yardstick for
    the fused passes: per slice a transmit, a cuFFT C2C forward transform, the propagator
    (band-limit and 1/N folded in) and a cuFFT inverse; then the lens the same way and
    |psi|^2 (torch.fft = cuFFT plus torch element-wise kernels).  Timed eagerly, L2
    flushed before every image; the result is checked against the fused image."""
    from emsim_gb300 import physics
    n, B, ns, d, kev = db.n1, db.B, db.ns, db.pixel, db.kev
    dev = db.slices.device
    lam = physics.electron_wave_length_angstrom(kev)
    gam = physics.electron_relativity_gamma(kev)
    sigma = float(np.float32(lam) * np.float32(gam))
    f = torch.fft.fftfreq(n, d=d, dtype=torch.float64, device=dev)
    f2 = f[:, None] ** 2 + f[None, :] ** 2
    keep = (f2 <= (0.6667 * 0.5 / d) ** 2).to(torch.float64)
    prop = (torch.polar(keep, -math.pi * lam * db.dz * f2) / (n * n)).to(torch.complex64)
    c1 = 0.5 * math.pi * db.cs_mm * 1e7 * lam ** 3
    c2 = math.pi * float(db.df[0]) * lam
    aper = (f2 <= (db.aperture / lam) ** 2).to(torch.float64)
    lens = (torch.polar(aper, -(c1 * f2 * f2 - c2 * f2)) / (n * n)).to(torch.complex64)
    amp = math.sqrt(db.dose * d * d)
    slices = db.slices

    def image():
        psi = torch.full((B, n, n), amp, dtype=torch.complex64, device=dev)
        for s_ in range(ns):
            psi = psi * torch.polar(torch.ones((), device=dev), sigma * slices[:, s_])
            psi = torch.fft.ifft2(torch.fft.fft2(psi) * prop, norm="forward")
        psi = torch.fft.ifft2(torch.fft.fft2(psi) * lens, norm="forward")
        return psi.real ** 2 + psi.imag ** 2

    t_plain = timed(torch, image, reps, flush)
    img = image()
    t_fused = timed(torch, db.run_image, reps, flush)
    ours = db.img
    rel = float(torch.linalg.vector_norm((img - ours).double()) / torch.linalg.vector_norm(ours.double()))
    return {"workload": f"multislice + lens + |psi|^2 of {B} stack(s) of {ns} slices, {n}^2",
            "design": "per slice: transmit, cuFFT C2C forward, propagate, cuFFT C2C inverse (torch.fft + "
                      "torch element-wise kernels); eager, L2 flushed",
            "plain_cufft_images_per_s": round(B / t_plain, 3), "fused_images_per_s": round(B / t_fused, 3),
            "speedup": round(t_plain / t_fused, 3), "rel_l2_plain_vs_fused": rel}


def graphs_extra(torch, n_mols: int = 4, reps: int = 20) -> dict:
    """Small batches through Pipe.run_batch(to_host=True), where launching is a large part
    of a call: n_mols blobs of the blob workload per call, eager launches against the
    CUDA graph that Pipe(cuda_graphs=True) replays for a structure seen before (both warm,
    wall clock per call, images checked bitwise equal)."""
    import time
    from emsim_gb300 import atoms, pipe, tem
    from emsim_gb300.synth import protein_blob
    W = BLOB
    mols = [atoms.AtomList(*protein_blob(W["n_atoms"], W["radius"], 500 + s)) for s in range(n_mols)]
    t_ = tem.TEM(electron_dose=W["dose"], beam_energy_kev=W["kev"], cs_mm=W["cs_mm"], defocus=W["defocus"],
                 aperture=W["aperture"])
    out = {"workload": f"{n_mols} blobs of the blob workload per Pipe.run_batch(to_host=True) call "
                       f"(roi {W['roi']}, 40 slices), wall clock per call"}
    imgs = {}
    for mode in ("eager", "cuda_graphs"):
        p = pipe.Pipe(t_, resolution=W["resolution"], slice_thickness=W["slice_thickness"], roi=W["roi"],
                      add_water=False, cuda_graphs=(mode == "cuda_graphs"))
        for _ in range(3):
            imgs[mode] = p.run_batch(mols, to_host=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            p.run_batch(mols, to_host=True)
        dt = (time.perf_counter() - t0) / reps
        out[mode] = {"images_per_s": round(n_mols / dt, 1), "ms_per_call": round(1e3 * dt, 3)}
    out["bitwise_equal"] = all(bool(np.array_equal(a, b)) for a, b in zip(imgs["eager"], imgs["cuda_graphs"]))
    return out


def batching_extra(torch, p, n_blobs: int = 256, reps: int = 2) -> dict:
    """The batching workload through Pipe.run_batch: 256 blobs with log-uniform 5k-200k
    atoms at 0.1 A^-3, random orientations, roi 256 or 512, every other one in amorphous
    ice; wall clock from host atoms to device images (ragged slice counts, two lateral
    sizes on two streams, two chunks)."""
    from emsim_gb300 import atoms, synth
    mix = synth.batching_mix(n_blobs, seed=11, pixel=0.5 * BLOB["resolution"])
    mols = [atoms.AtomList(el, xyz) for el, xyz, _ in mix]
    rois = [r for _, _, r in mix]
    p.run_batch(mols, rois=rois)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        p.run_batch(mols, rois=rois)
    torch.cuda.synchronize()
    dt = (time.perf_counter() - t0) / reps
    return {"workload": f"{n_blobs} blobs of the batching mix (5k-200k atoms log-uniform, 0.1 A^-3, random "
                        f"orientation, roi 256/512, half in ice), pixel 1 A, dz 2 A, one Pipe.run_batch call",
            "images_per_s": round(n_blobs / dt, 1), "seconds_per_batch": round(dt, 4),
            "atoms": int(sum(len(m.elements) for m in mols)), "roi_256": rois.count(256), "roi_512": rois.count(512),
            "timing": "wall clock from host AtomLists to device images (H2D included)"}


def read_traffic():
    """DRAM bytes per launch from the committed ncu summary (profiles/dram_traffic.txt)."""
    f = ROOT / "profiles" / "dram_traffic.txt"
    out = {}
    if f.exists():
        for line in f.read_text().splitlines():
            if line.startswith("#") or "=" not in line:
                continue
            k, v = line.split("=", 1)
            try:
                out[k.strip()] = float(v.split()[0])
            except ValueError:
                pass
    return out


# ---------------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------------
def run_ours(args):
    import torch
    import torch.distributed as dist

    rank, world, local = rank_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    from emsim_gb300 import atoms, autotune, backend, pipe, tem
    from emsim_gb300 import build as b
    b.build()

    # pass kernels and tiles picked by the autotuner for the sizes measured below
    tuned = {}
    if not args.no_tune:
        for n, nb in [(SLAB["n"], args.batch), (512, 32), (BLOB["roi"], 128)]:
            if args.tuning_from_cache:  # e.g. under a profiler, where timing the candidates is meaningless
                entry = autotune.ensure(n, n)
                if entry is None:
                    raise SystemExit(f"--tuning-from-cache: no cached tuning for {n}x{n} in {autotune.cache_path()}")
                tuned[f"{n}x{n}"] = entry
            else:
                tuned[f"{n}x{n}"] = autotune.tune(n, n, batch=nb, n_slices=6, reps=3)
    seed = 1000 * rank
    seeds = [seed + i for i in range(args.batch)]
    db = slab_step(torch, seeds)
    dev = torch.device("cuda", local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # warm-up (plans, propagator tables, lazy module loading)
    for _ in range(args.warmup):
        db.run()
    torch.cuda.synchronize()
    backend._native.check_device_error()
    graph = None if args.no_graph else db.graph()

    def step():
        if graph is not None:
            graph.replay()
        else:
            db.run()

    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    times = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.nvtx.range_push("timed")  # a profiler can capture exactly the timed steps
            e0.record()
            step()
            e1.record()
            torch.cuda.nvtx.range_pop()
            e1.synchronize()
            times.append(e0.elapsed_time(e1) * 1e-3)
    torch.cuda.synchronize()
    if backend._native.check_device_error() != 0:
        raise RuntimeError("a kernel's bounded wait gave up during the timed steps")
    t_total = float(sum(times))
    if world > 1:
        tt = torch.tensor([t_total], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_total = float(tt.item())
        dist.barrier()
    value = db.B * world * args.steps / t_total
    img_gpu = db.img[0].cpu().numpy()

    # ---- end to end through the public API (host atoms -> host image) ------------
    df, ap = scherzer()
    t_ = tem.TEM(electron_dose=SLAB["dose"], beam_energy_kev=SLAB["kev"], cs_mm=SLAB["cs_mm"], defocus=df,
                 aperture=ap)
    p = pipe.Pipe(t_, resolution=2 * SLAB["pixel"], slice_thickness=SLAB["dz"], roi=SLAB["n"], add_water=False)
    mols = [atoms.AtomList(*slab_atoms(s_)) for s_ in seeds]
    # atom offsets, float32 xyz and int32 Z of every molecule
    h2d = 4 * (len(mols) + 1) + sum(m.coordinates.astype(np.float32).nbytes + 4 * len(m.elements) for m in mols)
    e2e_steps = max(3, min(args.steps, 6))
    pe = pipelined_e2e(torch, p, mols, e2e_steps)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        host_serial = p.run_batch(mols, to_host=True)
    serial_value = len(mols) * e2e_steps / (time.perf_counter() - t0)
    same_api = all(bool(np.array_equal(x, y)) for x, y in zip(pe["host"], host_serial))
    same_step = bool(np.array_equal(pe["host"][0], img_gpu))
    e2e = {"value": pe["value"], "unit": "images/s", "h2d_bytes_per_step": int(h2d),
           "d2h_bytes_per_step": int(sum(x.nbytes for x in pe["host"])),
           "api": "emsim_gb300.pipe.Pipe.submit_batch / PendingImages.result (two batches in flight)",
           "timing": "wall clock over all steps: per step pinned staging of the host AtomLists, H2D, device "
                     "front-end, slices (built a few pairs at a time: the stacks exceed Pipe's 2 GiB limit), "
                     "images, one D2H of the images",
           "serial_run_batch": {"value": serial_value, "api": "emsim_gb300.pipe.Pipe.run_batch(to_host=True)"},
           "pipelined_equals_serial": same_api, "api_image_equals_device_step": same_step}

    if rank != 0 or args.headline_only:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": round(value, 3), "unit": "images/s", "n_gpus": world,
                              "steps": args.steps, "warmup": args.warmup, "config": dict(CONFIG),
                              "ms_per_step": round(1e3 * t_total / args.steps, 4), "e2e": e2e,
                              "note": "headline only (--headline-only)"}))
        if world > 1:
            dist.destroy_process_group()
        return

    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"

    # ---- roofline: slice step and slice build of the headline step ----------------
    rl_step = slice_step_on(torch, db, peak, flush=flush)
    rl_build = build_roofline(torch, db, peak, flush=flush)
    t_steps = rl_step["step_s"] * db.ns
    traffic = read_traffic()
    # the captured figures hold for the batch they were captured on (null for another)
    for key in ("slice_step_2048", "slice_build_2048"):
        if traffic.get(key + "_images") != db.B:
            traffic.pop(key, None)
    if t_steps >= rl_build["seconds"]:
        roofline = {"bound": "hbm", "kernel": "slice step = fused row pass + column pass (2048^2, %d images), "
                                              "averaged over the 400 steps of the headline step" % db.B,
                    "achieved": round(rl_step["achieved_gbs"], 1), "peak": peak, "unit": "GB/s",
                    "frac": round(rl_step["frac"], 4), "traffic": traffic.get("slice_step_2048"),
                    "peak_source": peak_src, "algorithmic_bytes_per_launch": rl_step["algorithmic_bytes"],
                    "seconds_per_launch": rl_step["step_s"]}
    else:
        roofline = {"bound": "hbm", "kernel": rl_build["kernel"], "achieved": round(rl_build["achieved_gbs"], 1),
                    "peak": peak, "unit": "GB/s", "frac": round(rl_build["frac"], 4),
                    "traffic": traffic.get("slice_build_2048"), "peak_source": peak_src,
                    "algorithmic_bytes_per_launch": rl_build["algorithmic_bytes"],
                    "seconds_per_launch": rl_build["seconds"]}
    step_parts = {"slice_build_s": round(rl_build["seconds"], 6), "slice_steps_s": round(t_steps, 6),
                  "slice_build_hbm_frac": round(rl_build["frac"], 4), "slice_step_hbm_frac": round(rl_step["frac"], 4),
                  "note": "component timings come from separate eager runs (L2 flushed) and can sum to slightly "
                          "more than the graphed step"}
    plain = plain_cufft_extra(torch, db, flush)
    step_images, launches = db.B, db.launches_per_step()
    del db
    torch.cuda.empty_cache()
    chunked = chunked_extra(torch, seed, flush)

    rl = {}
    for n, n_img, ns in [(256, 128, 40), (512, 32, 16), (2048, 2, 16)]:
        rl[n] = slice_step_roofline(torch, backend, n, n_img, ns, peak)
    diff_fwd = diff512_forward_extra(torch, flush)
    blob, bdb = blob_extra(torch, flush, max(3, min(args.steps, 10)), peak)
    blob_img0 = bdb.img[0].cpu().numpy()
    precision, img_bf16 = precision_extra(torch, bdb, backend, flush)
    del bdb
    torch.cuda.empty_cache()
    diff = differentiation_extra(torch)
    graphs = graphs_extra(torch)
    batching = batching_extra(torch, pipe.Pipe(
        tem.TEM(electron_dose=BLOB["dose"], beam_energy_kev=BLOB["kev"], cs_mm=BLOB["cs_mm"],
                defocus=BLOB["defocus"], aperture=BLOB["aperture"]),
        resolution=BLOB["resolution"], slice_thickness=BLOB["slice_thickness"], roi=BLOB["roi"], add_water=False))

    # ---- CPU baseline (the reference numpy algorithm on one core, a bounded sample of
    # the headline image) and the checker's FP64 image of the first blob -------------
    cpu = cpu_baseline(budget_s=args.cpu_seconds)
    acc = blob_accuracy(blob_img0, {"bf16x3": img_bf16})
    precision["bf16x3"].update(acc.pop("bf16x3", {}))

    clocks = clk.summary()
    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "images/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * t_total / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (complex64 waves)", "data": "synthetic (seeded slab)",
        "config": dict(CONFIG),
        "setup": {"images_per_step_per_gpu": step_images,
                  "l2": "flushed (256 MiB write) before every timed step; the %.1f GB of slice stacks are larger "
                        "than L2 too" % (step_images * 4.0 * SLAB["n_slices"] * SLAB["n"] ** 2 / 1e9),
                  "cuda_graph": graph is not None, "parallelism": f"image-parallel x{world}",
                  "autotune": {k: {"row": v["row"], "col": v["col"]} for k, v in tuned.items()}},
        "slice_steps_per_s": round(value * SLAB["n_slices"], 1),
        "step_parts": step_parts,
        "slice_step_throughput": {str(k): {"slice_steps_per_s": round(v["slice_steps_per_s"], 1),
                                           "hbm_frac": round(v["frac"], 4), "images": v["images"]}
                                  for k, v in rl.items()},
        "images_512_forward": diff_fwd,
        "blob_256": blob,
        "accuracy": {"blob_256": acc, "slab_2048": "tests/test_gpu_precision.py (FP64 oracle slab by slab)"},
        "precision": precision,
        "plain_cufft": plain,
        "chunked_slices": chunked,
        "differentiation": diff,
        "batching": batching,
        "api_cuda_graphs": graphs,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches * args.steps,
        "clocks": clocks,
    }
    print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


# ---------------------------------------------------------------------------------
# CPU reference: the oracle's bit-exact restatement of the reference numpy backend,
# timed on a bounded sample of the headline image
# ---------------------------------------------------------------------------------
_SLAB_STATE = {}


def _slab_state(seed: int):
    """Per-process state of the slab sample: atoms sorted by slice, the numpy-rule bin
    edges of the whole image, scattering factors, the numpy-semantics propagator and a
    running wave."""
    if seed in _SLAB_STATE:
        return _SLAB_STATE[seed]
    os.environ.setdefault("EMSIM_ORACLE_WORKERS", "1")
    from oracle import multislice as om
    el, xyz = slab_atoms(seed)
    xyz = om.centralize(xyz)
    n, ns, d, dz = SLAB["n"], SLAB["n_slices"], SLAB["pixel"], SLAB["dz"]
    edges = [om.numpy_bin_edges(ns, dz), om.numpy_bin_edges(n, d), om.numpy_bin_edges(n, d)]
    order = np.argsort(xyz[:, 0], kind="stable")
    xyz = xyz[order]
    zb = np.searchsorted(xyz[:, 0], edges[0])
    sf = om.scattering_factors_half([6], n, n, d, d)
    wp = om.WavePropagator(n, n, d, d, SLAB["kev"], "numpy")
    st = {"om": om, "xyz": xyz, "edges": edges, "zb": zb, "sf": sf, "wp": wp, "psi": wp.init_wave(SLAB["dose"]),
          "next": 0}
    _SLAB_STATE[seed] = st
    return st


def _slab_sample(k: int = 2, seed: int = 0):
    """k slices of the headline image through the reference numpy algorithm (numpy-rule
    binning of the slab's atoms on the image's own bin edges, make_multi_slices with the
    band-limit and clip, k multislice steps), then the lens and |psi|^2 of the wave.
    Returns (seconds per slice, seconds of the per-image lens + intensity)."""
    st = _slab_state(seed)
    om, wp = st["om"], st["wp"]
    df, ap = scherzer()
    s0 = st["next"]
    st["next"] = (s0 + k) % (SLAB["n_slices"] - k + 1)
    t0 = time.perf_counter()
    e = st["edges"]
    pts = st["xyz"][st["zb"][s0]:st["zb"][s0 + k]]
    hist, _ = np.histogramdd(pts, bins=[e[0][s0:s0 + k + 1], e[1], e[2]])
    hist = np.ascontiguousarray(hist[None], dtype=np.float32)
    slices = om.make_slices(hist, st["sf"], "numpy")
    st["psi"] = wp.multislice_propagate(st["psi"], slices, SLAB["dz"])
    t1 = time.perf_counter()
    om.intensity(wp.lens_propagate(st["psi"], SLAB["cs_mm"], df, ap))
    t2 = time.perf_counter()
    return (t1 - t0) / k, t2 - t1


def _slab_images_per_s(samples, procs: int) -> float:
    """Images/s of procs processes that each take t_slice per slice and t_lens per image:
    one image = 400 slices + one lens and intensity."""
    ts = float(np.median([s[0] for s in samples]))
    tl = float(np.median([s[1] for s in samples]))
    return procs / (SLAB["n_slices"] * ts + tl)


def cpu_baseline(budget_s: float = 15.0) -> dict:
    """Images/s of the reference numpy algorithm on one host core, from a bounded sample
    of the headline image (2 slices per round plus the lens, scaled to 400 slices)."""
    _slab_sample()  # state + warm
    t0 = time.perf_counter()
    samples = []
    while time.perf_counter() - t0 < budget_s or not samples:
        samples.append(_slab_sample())
    dt = time.perf_counter() - t0
    v = _slab_images_per_s(samples, 1)
    return {"value": round(v, 6), "unit": "images/s", "cores": 1, "kind": "port",
            "sample": f"{2 * len(samples)} of the headline image's 400 slices (numpy-rule binning, "
                      f"make_multi_slices, multislice) and {len(samples)} lens + |psi|^2 through the reference "
                      f"numpy algorithm (oracle 'numpy' semantics, bit-exact with emsim's numpy backend, "
                      f"complex128, numpy FFT) in {dt:.1f} s; images/s = 1 / (400 t_slice + t_lens)"}


def blob_accuracy(img, others=None) -> dict:
    """Relative L2 errors of the first blob's GPU images against the FP64 oracle."""
    from oracle import multislice as om
    from emsim_gb300.synth import protein_blob
    W = BLOB
    el, xyz = protein_blob(W["n_atoms"], W["radius"], 0)
    ref64 = om.pipe_run(el, xyz, resolution=W["resolution"], slice_thickness=W["slice_thickness"], roi=W["roi"],
                        beam_energy_kev=W["kev"], dose=W["dose"], cs_mm=W["cs_mm"], defocus=W["defocus"],
                        aperture=W["aperture"], semantics="fftw", dtype=np.float64)

    def errs(x):
        return {"rel_l2_image_vs_fp64": om.rel_l2(x, ref64),
                "rel_l2_contrast_vs_fp64": om.rel_l2(x - x.mean(), ref64 - ref64.mean())}

    acc = errs(img)
    for name, other in (others or {}).items():
        if other is not None:
            acc[name] = errs(other)
    return acc


def _ref_step(i: int):
    return _slab_sample(2, seed=0)


def run_reference(args):
    rank, world, _ = rank_env()
    if rank != 0:
        return
    import multiprocessing as mp
    procs = os.cpu_count() or 1
    ctx = mp.get_context("spawn")
    samples = []
    t_wall = []
    with ctx.Pool(procs) as pool:
        pool.map(_ref_step, range(procs))  # per-process state and a warm call
        for _ in range(args.warmup):
            pool.map(_ref_step, range(procs))
        for _ in range(args.steps):
            t0 = time.perf_counter()
            samples.extend(pool.map(_ref_step, range(procs)))
            t_wall.append(time.perf_counter() - t0)
    v = _slab_images_per_s(samples, procs)
    out = {"impl": "reference", "metric": METRIC, "value": round(v, 6), "unit": "images/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64 (numpy complex128)", "data": "synthetic (seeded slab)",
           "config": dict(CONFIG),
           "setup": {"parallelism": f"{procs} host processes"},
           "ms_per_step": round(1e3 * float(np.median(t_wall)), 3),
           "cpu_baseline": {"value": round(v, 6), "unit": "images/s", "cores": procs, "kind": "port",
                            "sample": f"per step, each of {procs} processes runs 2 of the headline image's 400 "
                                      f"slices (numpy-rule binning, make_multi_slices, multislice) and one lens + "
                                      f"|psi|^2 through the reference numpy algorithm (bit-exact oracle "
                                      f"restatement; the reference tree is not present on the GPU host); "
                                      f"images/s = processes / (400 t_slice + t_lens), medians over "
                                      f"{len(samples)} samples"},
           "e2e": {"value": round(v, 6), "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--batch", type=int, default=8, help="slab images per step (seeds rank*1000 + 0..batch-1)")
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
    ap.add_argument("--headline-only", action="store_true",
                    help="time the headline step and its end-to-end figure only (for profiler runs)")
    ap.add_argument("--tuning-from-cache", action="store_true",
                    help="apply the cached autotuner choice instead of measuring it")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
