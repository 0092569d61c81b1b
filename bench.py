"""Throughput benchmark of the emsim multislice hot path on GB300.

Workload (one step): a batch of protein-like blobs, each 50,000 C/N/O/S atoms
(fractions 0.63/0.17/0.19/0.01, seeded) uniform in a 40 A sphere, imaged at roi 256,
resolution 2 A (pixel 1 A), slice thickness 2 A (40 slices), 200 keV, Cs 1.3 mm,
defocus 700 A, aperture 10 mrad, plain FP32: atom binning -> projected-potential
slices -> multislice -> lens -> |psi|^2.  Inputs are resident in HBM for ``value``;
``e2e`` runs the same images through the public ``Pipe.submit_batch`` API (two
batches in flight) from host atoms to host images, every step copying its atoms in and
its images out.  L2 is flushed (256 MiB write) before every timed step; each step is timed
with CUDA events on the launching stream.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--batch B] [--impl reference]

Multi-GPU (torchrun): every rank images its own blobs (weak scaling, no collective on
the data path); rank 0 prints the max-over-ranks time.
"""
from __future__ import annotations

import argparse
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

WORKLOAD = dict(n_atoms=50_000, radius=40.0, roi=256, resolution=2.0, slice_thickness=2.0, kev=200.0,
                cs_mm=1.3, defocus=700.0, aperture=10e-3, dose=20.0)
METRIC = "images/s (50k-atom blob, 256^2, 40 slices, plain FP32)"


def blob(seed: int):
    from emsim_gb300.synth import protein_blob  # seeded synthetic input generator
    return protein_blob(WORKLOAD["n_atoms"], WORKLOAD["radius"], seed)


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


# ---------------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------------
class DeviceBatch:
    """Device-resident inputs and buffers for B blobs; run() queues one full step:
    slices of all blobs straight from their atoms (one call), then plane wave ->
    multislice -> lens -> |psi|^2 for all blobs (one call)."""

    def __init__(self, seeds, torch, backend, atoms, pot):
        W = WORKLOAD
        self.torch = torch
        self.backend = backend
        dev = torch.device("cuda", torch.cuda.current_device())
        pix = 0.5 * W["resolution"]
        self.pix = pix
        geo = []
        for s in seeds:
            el, xyz = blob(s)
            mol = atoms.centralize(atoms.AtomList(el, xyz))
            mol, uz, cnt = atoms.sort_elements_and_count(mol)
            ns, n1, n2 = pot.finalize_slice_size(tuple(mol.space), (pix, pix), W["slice_thickness"], W["roi"], None)
            geo.append((mol.coordinates, tuple(int(z) for z in uz), cnt, ns))
        keys = {(g[1], g[3]) for g in geo}
        if len(keys) != 1:
            raise RuntimeError(f"blobs of one batch need equal elements and slice counts, got {sorted(keys)}")
        (uz, ns), = keys
        self.ns = ns
        self.n = W["roi"]
        self.B = len(seeds)
        self.builder = backend.MultiSlicesBuilder(list(uz), ns, self.n, self.n, W["slice_thickness"], pix, pix)
        xyz = np.ascontiguousarray(np.concatenate([g[0] for g in geo]))
        counts = np.stack([g[2] for g in geo]).astype(np.uint32)
        self.n_atoms = int(xyz.shape[0])
        self.coords = torch.from_numpy(xyz).to(dev)
        self.counts = torch.from_numpy(counts.view(np.int32)).to(dev)
        self.slices = torch.empty((self.B, ns, self.n, self.n), dtype=torch.float32, device=dev)
        self.work = torch.empty((self.B, self.n, self.n), dtype=torch.complex64, device=dev)
        self.img = torch.empty((self.B, self.n, self.n), dtype=torch.float32, device=dev)
        lib = backend._native.load()
        self.ws_bytes = int(lib.emsim_gb300_build_slices_workspace_size(self.builder._plan.handle, self.n_atoms,
                                                                       self.B))
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=dev)
        self.wp = backend.WavePropagator(self.n, self.n, pix, pix, W["kev"])
        self.df = np.full(self.B, W["defocus"], dtype=np.float64)

    def launches_per_step(self) -> int:
        # slices: group scan (2) + bucket + bucket scan (3) + scatter + column pass + row pass
        slices = 2 + 1 + 3 + 1 + 2
        lens = math.ceil(self.B / 64)
        return slices + 2 * self.ns + lens + 1

    def run(self):
        import ctypes
        nat = self.backend._native
        st = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        P = self.backend._ptr
        nat.call("emsim_gb300_build_slices", self.builder._plan.handle, P(self.coords), self.n_atoms,
                 P(self.counts), self.B, P(self.slices), P(self.ws), self.ws_bytes, st)
        self.run_image()

    def run_image(self):
        """plane wave -> multislice -> lens -> |psi|^2 of all blobs from the built slices."""
        import ctypes
        nat = self.backend._native
        st = ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)
        P = self.backend._ptr
        W = WORKLOAD
        nat.call("emsim_gb300_multislice_image", self.wp._plan.handle, P(self.slices), self.ns,
                 self.ns * self.n * self.n, W["slice_thickness"], W["dose"], W["cs_mm"],
                 self.df.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), self.B, W["aperture"], P(self.img),
                 P(self.work), None, self.B, st)


def slice_step_roofline(torch, backend, n: int, n_img: int, n_slices: int, peak_gbs: float, reps: int = 5):
    """Average duration of one slice step (fused row pass + column pass) on a batch of
    n_img waves of n x n, from CUDA events around multislice_propagate calls."""
    dev = torch.device("cuda", torch.cuda.current_device())
    wp = backend.WavePropagator(n, n, 0.5, 0.5, 200.0)
    w = torch.ones((n_img, n, n), dtype=torch.complex64, device=dev)
    sl = torch.rand((n_img, n_slices, n, n), dtype=torch.float32, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    for _ in range(2):
        wp.multislice_propagate(w, sl, 2.0)
    ts = []
    for _ in range(reps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        wp.multislice_propagate(w, sl, 2.0)
        e1.record()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t = float(np.median(ts))
    # n_slices steps + one final row pass (the inverse rows of the exit wave)
    per_step = t / (n_slices + 0.5)
    algo = 20.0 * n * n * n_img  # bytes per slice step: psi read 8 + psi write 8 + V read 4
    return {"n": n, "images": n_img, "slices": n_slices, "step_s": per_step,
            "slice_steps_per_s": n_img / per_step, "achieved_gbs": algo / per_step / 1e9,
            "frac": algo / per_step / 1e9 / peak_gbs}


def slice_build_roofline(torch, db, peak_gbs: float, reps: int = 5) -> dict:
    """The histogram-free slice build of the bench step (emsim_gb300_build_slices for all
    its blobs) timed alone with CUDA events, L2 flushed, against its algorithmic bytes:
    16 B per atom read (float32 xyz + the element counts' share) and 4 B per slice pixel
    written.  The kernel is issue-bound on FFT arithmetic, not on these bytes."""
    import ctypes
    nat = db.backend._native
    P = db.backend._ptr
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=db.slices.device)

    def build():
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        nat.call("emsim_gb300_build_slices", db.builder._plan.handle, P(db.coords), db.n_atoms, P(db.counts), db.B,
                 P(db.slices), P(db.ws), db.ws_bytes, st)

    build()
    ts = []
    for _ in range(reps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        build()
        e1.record()
        e1.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    t = float(np.median(ts))
    algo = 16.0 * db.n_atoms + 4.0 * db.B * db.ns * db.n * db.n
    return {"bound": "hbm", "kernel": "slice build = bucketing + slice_cols_atoms_kernel + slice_rows_inv_kernel "
                                      "(%d blobs, %d slices of %d^2)" % (db.B, db.ns, db.n),
            "achieved": round(algo / t / 1e9, 1), "peak": peak_gbs, "unit": "GB/s",
            "frac": round(algo / t / 1e9 / peak_gbs, 4), "seconds": round(t, 6),
            "algorithmic_bytes_per_launch": algo,
            "note": "issue-bound on the 4 + 1 column FFTs and the fixed-point row sums per slice pair"}


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


def precision_extra(torch, db, backend, flush, reps: int = 5):
    """The bench step (eager launches, L2 flushed) with the multislice passes in FP32 and in
    split-BF16 on the tensor cores; returns the timing dict and the split-BF16 image of the
    first blob (its accuracy against FP64 is computed in the CPU leg)."""
    out, img = {}, None
    try:
        for mode in ("fp32", "bf16x3"):
            backend.set_precision(mode)
            for _ in range(2):
                db.run()
            times = []
            for _ in range(reps):
                flush.fill_(1.0)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                db.run()
                e1.record()
                e1.synchronize()
                times.append(e0.elapsed_time(e1) * 1e-3)
            out[mode] = {"images_per_s": round(db.B * reps / float(sum(times)), 1)}
            if mode == "bf16x3":
                img = db.img[0].cpu().numpy()
    finally:
        backend.set_precision("fp32")
    out["workload"] = "the bench step, eager launches (no CUDA graph), L2 flushed before every step"
    out["bf16x3_passes"] = ("256-point row pass (IFFT, transmit, FFT) and column pass (FFT, propagate, IFFT) as "
                            "16x16 four-step DFTs on tcgen05, bf16 hi+lo operands, fp32 accumulation")
    return out, img


def plain_cufft_extra(torch, db, backend, flush, reps: int = 3) -> dict:
    """The reference's CUDA design on the same GPU and the same slices, as a yardstick for
    the fused passes: per slice a transmit, a cuFFT C2C forward transform, the propagator
    (band-limit and 1/N folded in) and a cuFFT inverse; then the lens the same way and
    |psi|^2 (torch.fft = cuFFT plus torch element-wise kernels).  Timed eagerly, L2
    flushed before every step; the result is checked against the fused image."""
    from emsim_gb300 import physics
    W = WORKLOAD
    n, B, ns, d = db.n, db.B, db.ns, db.pix
    dev = db.slices.device
    lam = physics.electron_wave_length_angstrom(W["kev"])
    gam = physics.electron_relativity_gamma(W["kev"])
    sigma = float(np.float32(lam) * np.float32(gam))
    f = torch.fft.fftfreq(n, d=d, dtype=torch.float64, device=dev)
    f2 = f[:, None] ** 2 + f[None, :] ** 2
    fmax = 0.5 / d
    keep = (f2 <= (0.6667 * fmax) ** 2).to(torch.float64)
    prop = (torch.polar(keep, -math.pi * lam * W["slice_thickness"] * f2) / (n * n)).to(torch.complex64)
    c1 = 0.5 * math.pi * W["cs_mm"] * 1e7 * lam ** 3
    c2 = math.pi * W["defocus"] * lam
    aper = (f2 <= (W["aperture"] / lam) ** 2).to(torch.float64)
    lens = (torch.polar(aper, -(c1 * f2 * f2 - c2 * f2)) / (n * n)).to(torch.complex64)
    amp = math.sqrt(W["dose"] * d * d)
    slices = db.slices

    def image():
        psi = torch.full((B, n, n), amp, dtype=torch.complex64, device=dev)
        for s_ in range(ns):
            psi = psi * torch.polar(torch.ones((), device=dev), sigma * slices[:, s_])
            psi = torch.fft.ifft2(torch.fft.fft2(psi) * prop, norm="forward")
        psi = torch.fft.ifft2(torch.fft.fft2(psi) * lens, norm="forward")
        return psi.real ** 2 + psi.imag ** 2

    for _ in range(2):
        img = image()
    times = []
    for _ in range(reps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        img = image()
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    ours = db.img
    rel = float(torch.linalg.vector_norm((img - ours).double()) / torch.linalg.vector_norm(ours.double()))
    # our fused image call on the same slices, timed the same way, in both precisions
    fused = {}
    try:
        for mode in ("fp32", "bf16x3"):
            backend.set_precision(mode)
            db.run_image()
            tf = []
            for _ in range(reps):
                flush.fill_(1.0)
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                db.run_image()
                e1.record()
                e1.synchronize()
                tf.append(e0.elapsed_time(e1) * 1e-3)
            fused[mode] = round(B * reps / float(sum(tf)), 1)
    finally:
        backend.set_precision("fp32")
    return {"workload": f"multislice + lens + |psi|^2 of the bench step's {B} stacks of {ns} slices, {n}^2",
            "design": "per slice: transmit, cuFFT C2C forward, propagate, cuFFT C2C inverse (torch.fft + "
                      "torch element-wise kernels); eager, L2 flushed",
            "plain_cufft_images_per_s": round(B * reps / float(sum(times)), 1),
            "fused_fp32_images_per_s": fused["fp32"], "fused_bf16x3_images_per_s": fused["bf16x3"],
            "rel_l2_plain_vs_fused": rel}


def batching_extra(torch, p, n_blobs: int = 32, reps: int = 2) -> dict:
    """A mixed batch through Pipe.run_batch: blobs with log-uniform 5k-200k atoms at
    0.1 A^-3, random orientations, roi 256 or 512, every other one in amorphous ice;
    wall clock from host atoms to device images (ragged slice counts, two lateral sizes
    on two streams)."""
    from emsim_gb300 import atoms, synth
    mix = synth.batching_mix(n_blobs, seed=11, pixel=0.5 * WORKLOAD["resolution"])
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


def run_ours(args):
    import torch
    import torch.distributed as dist

    rank, world, local = rank_env()
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    from emsim_gb300 import atoms, backend, pipe, pot, tem
    from emsim_gb300 import build as b
    b.build()

    B = args.batch
    seeds = [1000 * rank + i for i in range(B)]
    # pass kernels and tiles picked by the autotuner for the sizes measured below
    from emsim_gb300 import autotune
    tuned = {}
    if not args.no_tune:
        for n, nb in [(WORKLOAD["roi"], B), (512, 32), (2048, 2)]:
            if args.tuning_from_cache:  # e.g. under a profiler, where timing the candidates is meaningless
                entry = autotune.ensure(n, n)
                if entry is None:
                    raise SystemExit(f"--tuning-from-cache: no cached tuning for {n}x{n} in {autotune.cache_path()}")
                tuned[f"{n}x{n}"] = entry
            else:
                tuned[f"{n}x{n}"] = autotune.tune(n, n, batch=nb, n_slices=6, reps=3)
    db = DeviceBatch(seeds, torch, backend, atoms, pot)
    dev = torch.device("cuda", local)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    # warm-up (plans, propagator tables, lazy module loading)
    for _ in range(args.warmup):
        db.run()
    torch.cuda.synchronize()
    graph = None
    if not args.no_graph:
        s = torch.cuda.Stream()
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=s):
                db.run()
        torch.cuda.current_stream().wait_stream(s)
        graph.replay()
        torch.cuda.synchronize()

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
    t_total = float(sum(times))
    if world > 1:
        tt = torch.tensor([t_total], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_total = float(tt.item())
        dist.barrier()
    value = B * world * args.steps / t_total

    # ---- end to end through the public API (host atoms -> host image) ----------
    W = WORKLOAD
    t_ = tem.TEM(electron_dose=W["dose"], beam_energy_kev=W["kev"], cs_mm=W["cs_mm"], defocus=W["defocus"],
                 aperture=W["aperture"])
    p = pipe.Pipe(t_, resolution=W["resolution"], slice_thickness=W["slice_thickness"], roi=W["roi"],
                  add_water=False)
    mols = []
    h2d = 4 * (len(seeds) + 1)  # atom offsets
    for s in seeds:
        el, xyz = blob(s)
        mols.append(atoms.AtomList(el, xyz))
        h2d += xyz.astype(np.float32).nbytes + 4 * len(el)  # float32 coordinates + int32 Z
    for _ in range(2):
        p.run_batch(mols, to_host=True)
    torch.cuda.synchronize()
    e2e_steps = max(3, min(args.steps, 10))

    def e2e_run(pipelined: bool):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if pipelined:
            # the next step's host side (staging, H2D, front-end, launches) overlaps this
            # step's device work; every step still copies its atoms in and its images out
            pending = p.submit_batch(mols)
            for _ in range(e2e_steps - 1):
                following = p.submit_batch(mols)
                host = pending.result()
                pending = following
            host = pending.result()
        else:
            for _ in range(e2e_steps):
                host = p.run_batch(mols, to_host=True)
        torch.cuda.synchronize()
        return len(mols) * e2e_steps / (time.perf_counter() - t0), host

    e2e_run(True)
    e2e_value, host = e2e_run(True)
    serial_value, host_serial = e2e_run(False)
    same = all(np.array_equal(a, b) for a, b in zip(host, host_serial))
    e2e = {"value": e2e_value, "unit": "images/s", "h2d_bytes_per_step": h2d,
           "d2h_bytes_per_step": int(sum(x.nbytes for x in host)),
           "api": "emsim_gb300.pipe.Pipe.submit_batch / PendingImages.result (two batches in flight)",
           "timing": "wall clock over all steps: per step pinned staging of host AtomLists, H2D, device "
                     "front-end, slices, images, one D2H of the images",
           "serial_run_batch": {"value": serial_value, "api": "emsim_gb300.pipe.Pipe.run_batch(to_host=True)"},
           "pipelined_equals_serial": bool(same)}

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    img0 = db.img[0].cpu().numpy()
    plain = plain_cufft_extra(torch, db, backend, flush)
    precision, img_bf16 = precision_extra(torch, db, backend, flush)
    diff = differentiation_extra(torch)
    batching = batching_extra(torch, p)

    # ---- roofline of the dominant kernel pair (slice step) ----------------------
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    rl = {}
    for n, n_img, ns in [(256, B, db.ns), (512, 32, 16), (2048, 2, 16)]:
        rl[n] = slice_step_roofline(torch, backend, n, n_img, ns, peak)
    traffic = read_traffic()
    rl_build = slice_build_roofline(torch, db, peak)
    main = rl[256]
    roofline = {"bound": "hbm", "kernel": "slice step = row pass + column pass as tuned (256^2, batch %d)" % B,
                "achieved": round(main["achieved_gbs"], 1), "peak": peak, "unit": "GB/s",
                "frac": round(main["frac"], 4), "traffic": traffic.get("slice_step_256"),
                "peak_source": peak_src, "algorithmic_bytes_per_launch": 20 * 256 * 256 * B}

    # ---- CPU baseline: the oracle's restatement of the reference numpy path, and the
    # checker's FP64 image of the first benched blob ------------------------------
    cpu, acc = cpu_baseline(budget_s=args.cpu_seconds, check=(seeds[0], img0, {"bf16x3": img_bf16}))
    precision["bf16x3"].update(acc.pop("bf16x3", {}))

    clocks = clk.summary()
    out = {
        "metric": METRIC, "value": round(value, 2), "unit": "images/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1e3 * t_total / args.steps, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (complex64 waves)", "data": "synthetic (seeded blobs)",
        "config": {"workload": "blob 50k C/N/O/S atoms r=40A, roi 256, pixel 1A, dz 2A, %d slices, 200 keV, "
                               "Cs 1.3 mm, df 700 A, aperture 10 mrad" % db.ns,
                   "images_per_step_per_gpu": B, "l2": "flushed (256 MiB write) before every timed step",
                   "cuda_graph": graph is not None, "parallelism": f"image-parallel x{world}",
                   "autotune": {k: {"row": v["row"], "col": v["col"]} for k, v in tuned.items()}},
        "slice_steps_per_s": round(value * db.ns, 1),
        "slice_step_throughput": {str(k): {"slice_steps_per_s": round(v["slice_steps_per_s"], 1),
                                           "hbm_frac": round(v["frac"], 4), "images": v["images"]}
                                  for k, v in rl.items()},
        "accuracy": acc,
        "precision": precision,
        "plain_cufft": plain,
        "differentiation": diff,
        "batching": batching,
        "roofline": roofline,
        "roofline_slice_build": rl_build,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": db.launches_per_step() * args.steps,
        "clocks": clocks,
    }
    print(json.dumps(out))
    if world > 1:
        dist.destroy_process_group()


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
# CPU reference: the oracle's bit-exact restatement of the reference numpy backend
# ---------------------------------------------------------------------------------
def _cpu_one(seed: int) -> float:
    os.environ.setdefault("EMSIM_ORACLE_WORKERS", "1")
    from oracle import multislice as om
    W = WORKLOAD
    el, xyz = blob(seed)
    t0 = time.perf_counter()
    om.pipe_run(el, xyz, resolution=W["resolution"], slice_thickness=W["slice_thickness"], roi=W["roi"],
                beam_energy_kev=W["kev"], dose=W["dose"], cs_mm=W["cs_mm"], defocus=W["defocus"],
                aperture=W["aperture"], semantics="numpy")
    return time.perf_counter() - t0


def cpu_baseline(budget_s: float = 15.0, processes: int = 1, check=None):
    """Images/s of the reference numpy algorithm on host cores (bounded sample).  With
    ``check`` = (seed, GPU image, {name: other GPU image of the same blob}), also the
    relative L2 errors of those images against the FP64 oracle (outside the timed sample);
    returns (baseline, accuracy) then."""
    import multiprocessing as mp
    t0 = time.perf_counter()
    n = 0
    if processes <= 1:
        while time.perf_counter() - t0 < budget_s or n == 0:
            _cpu_one(n)
            n += 1
        dt = time.perf_counter() - t0
    else:
        ctx = mp.get_context("spawn")
        with ctx.Pool(processes) as pool:
            pool.map(_cpu_one, range(processes))  # import + warm
            t0 = time.perf_counter()
            rounds = 0
            while time.perf_counter() - t0 < budget_s or rounds == 0:
                pool.map(_cpu_one, range(processes))
                rounds += 1
            dt = time.perf_counter() - t0
            n = rounds * processes
    base = {"value": round(n / dt, 4), "unit": "images/s", "cores": processes, "kind": "port",
            "sample": f"{n} image(s) of the bench workload through the reference numpy algorithm "
                      f"(oracle 'numpy' semantics, bit-exact with emsim's numpy backend, complex128, "
                      f"numpy FFT) in {dt:.1f} s"}
    if check is None:
        return base
    from oracle import multislice as om
    W = WORKLOAD
    seed, img, others = check
    el, xyz = blob(seed)
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
    return base, acc


def run_reference(args):
    rank, world, _ = rank_env()
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    budget = max(5.0, args.cpu_seconds)
    vals = []
    for _ in range(args.warmup):
        _cpu_one(0)
    for k in range(args.steps):
        c = cpu_baseline(budget_s=budget / max(1, args.steps), processes=procs)
        vals.append(c["value"])
    v = float(np.median(vals))
    out = {"impl": "reference", "metric": METRIC, "value": round(v, 4), "unit": "images/s", "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64 (numpy complex128)", "data": "synthetic (seeded blobs)",
           "config": {"workload": "blob 50k C/N/O/S atoms r=40A, roi 256, pixel 1A, dz 2A, 40 slices, 200 keV, "
                                  "Cs 1.3 mm, df 700 A, aperture 10 mrad",
                      "parallelism": f"{procs} host processes"},
           "cpu_baseline": {"value": round(v, 4), "unit": "images/s", "cores": procs, "kind": "port",
                            "sample": "reference numpy algorithm (bit-exact oracle restatement; the reference "
                                      "tree is not present on the GPU host), one image per process per round"},
           "e2e": {"value": round(v, 4), "unit": "images/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--batch", type=int, default=128)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-graph", action="store_true")
    ap.add_argument("--no-tune", action="store_true")
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
