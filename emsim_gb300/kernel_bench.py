"""Micro-benchmark of the engine's hot calls on synthetic device-resident data.

Times one C-ABI call (median of --reps, CUDA events on the launching stream, L2
flushed before each rep) and prints a JSON line.  Also the small, bounded driver for
ncu captures of single kernels.

  python -m emsim_gb300.kernel_bench --case step  --n 512 --batch 64 --slices 4
  python -m emsim_gb300.kernel_bench --case slices --n 256 --elements 4 --slices 40
  python -m emsim_gb300.kernel_bench --case bin   --n 256 --slices 40 --atoms 50000

cases: step (multislice_propagate), space (space_propagate), lens (lens_propagate),
image (multislice_image: plane wave -> slices -> lens -> |psi|^2), slices
(make_multi_slices), atoms (build_slices: slices straight from atoms, --atoms per image,
uniform over the slab), blobs (build_slices of --batch seeded protein-like blobs of --atoms
atoms in a 40 A sphere), bin (bin_atoms_multi_slices), slab (the amorphous-carbon slab of the
bench's headline, 0.1 A^-3 C over --n x 0.1 A square, --slices slices of 0.5 A deep:
build_slices straight from its atoms, then multislice_image at 300 keV, Cs 1.0 mm, Scherzer).
"""
from __future__ import annotations

import argparse
import ctypes
import json

import numpy as np
import torch

from . import _native, backend


def _time(fn, reps: int, flush: torch.Tensor) -> float:
    """Median seconds per call; the timed calls sit in the NVTX range "timed" so that a
    profiler can capture exactly them."""
    ts = []
    for _ in range(reps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("timed")
        e0.record()
        fn()
        e1.record()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        ts.append(e0.elapsed_time(e1) * 1e-3)
    return float(np.median(ts))


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="step",
                    choices=["step", "space", "lens", "image", "slices", "atoms", "blobs", "bin", "slab"])
    ap.add_argument("--n", type=int, default=512)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--slices", type=int, default=4)
    ap.add_argument("--elements", type=int, default=4)
    ap.add_argument("--atoms", type=int, default=50000)
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=2)
    ap.add_argument("--autotune", action="store_true", help="tune the pass kernels for --n first")
    ap.add_argument("--tuning-from-cache", action="store_true", help="apply the cached tuning for --n")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "bf16x3"])
    args = ap.parse_args(argv)
    dev = torch.device("cuda", torch.cuda.current_device())
    torch.manual_seed(0)
    n, B, S = args.n, args.batch, args.slices
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    st = lambda: ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)  # noqa: E731
    P = backend._ptr
    out = {"case": args.case, "n": n, "precision": args.precision}
    backend.set_precision(args.precision)
    if args.autotune or args.tuning_from_cache:
        from . import autotune
        out["tuning"] = autotune.ensure(n, n) if args.tuning_from_cache else autotune.tune(n, n, batch=B)
        if out["tuning"] is None:
            raise SystemExit(f"no cached tuning for {n}x{n} in {autotune.cache_path()}")
    if args.case in ("step", "space", "lens", "image"):
        wp = backend.WavePropagator(n, n, 0.5, 0.5, 200.0)
        w = torch.ones((B, n, n), dtype=torch.complex64, device=dev)
        o = torch.empty_like(w)
        sl = torch.rand((B, S, n, n), dtype=torch.float32, device=dev)
        img = torch.empty((B, n, n), dtype=torch.float32, device=dev)
        df = np.full(B, 700.0)
        h = wp._plan.handle
        calls = {
            "step": lambda: _native.call("emsim_gb300_multislice_propagate", h, P(w), P(sl), S, S * n * n, 2.0, P(o),
                                         B, st()),
            "space": lambda: _native.call("emsim_gb300_space_propagate", h, P(w), 2.0, P(o), B, st()),
            "lens": lambda: _native.call("emsim_gb300_lens_propagate", h, P(w), 1.3, 700.0, 0.01, P(o), B, st()),
            "image": lambda: _native.call("emsim_gb300_multislice_image", h, P(sl), S, S * n * n, 2.0, 20.0, 1.3,
                                          df.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), B, 0.01, P(img),
                                          P(o), None, B, st()),
        }
        fn = calls[args.case]
        for _ in range(args.warmup):
            fn()
        t = _time(fn, args.reps, flush)
        px = B * n * n
        out.update(batch=B, slices=S, seconds=t)
        if args.case == "step":
            steps = S + 0.5
            out.update(slice_steps_per_s=B * S / t, algo_gbs=20.0 * px * S / t / 1e9,
                       moved_gbs_two_pass=(36.0 * px * S + 16.0 * px) / t / 1e9, per_step_us=1e6 * t / steps)
        elif args.case in ("space", "lens"):
            out.update(algo_gbs=16.0 * px / t / 1e9)
        else:
            out.update(images_per_s=B / t)
    elif args.case == "slices":
        E = args.elements
        zs = [6, 7, 8, 16, 1, 29][:E]
        b = backend.MultiSlicesBuilder(zs, S, n, n, 2.0, 1.0, 1.0)
        hist = torch.poisson(torch.full((E, S, n, n), 0.05, device=dev))
        o = torch.empty((S, n, n), dtype=torch.float32, device=dev)
        nbytes = int(_native.load().emsim_gb300_make_slices_workspace_size(b._plan.handle))
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        fn = lambda: _native.call("emsim_gb300_make_slices", b._plan.handle, P(hist), P(o), P(ws), nbytes,  # noqa
                                  st())
        for _ in range(args.warmup):
            fn()
        t = _time(fn, args.reps, flush)
        out.update(elements=E, slices=S, seconds=t, slices_per_s=S / t,
                   algo_gbs=(4.0 * E + 4.0) * S * n * n / t / 1e9)
    elif args.case == "blobs":
        # the bench's workload: --batch seeded 50k-atom C/N/O/S blobs (40 A sphere), each
        # centralised and sized as Pipe does (roi --n, pixel 1 A, 2 A slices)
        from . import atoms as atm
        from . import pot, synth
        geo = []
        for seed in range(B):
            mol = atm.centralize(atm.AtomList(*synth.protein_blob(args.atoms, 40.0, seed)))
            mol, uz, cnt = atm.sort_elements_and_count(mol)
            ns, _, _ = pot.finalize_slice_size(tuple(mol.space), (1.0, 1.0), 2.0, (n, n), None)
            geo.append((mol.coordinates, [int(z) for z in uz], cnt, ns))
        if any(g[1] != geo[0][1] for g in geo):
            raise SystemExit("blobs case: the seeded blobs need one element set")
        S = max(g[3] for g in geo)
        b = backend.MultiSlicesBuilder(geo[0][1], S, n, n, 2.0, 1.0, 1.0)
        xyz = np.ascontiguousarray(np.concatenate([g[0] for g in geo]).astype(np.float32))
        counts = np.stack([np.asarray(g[2]) for g in geo]).astype(np.uint32)
        N = int(xyz.shape[0])
        c = torch.from_numpy(xyz).to(dev)
        cn = torch.from_numpy(counts.view(np.int32)).to(dev)
        o = torch.empty((B, S, n, n), dtype=torch.float32, device=dev)
        nbytes = int(_native.load().emsim_gb300_build_slices_workspace_size(b._plan.handle, N, B))
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        fn = lambda: _native.call("emsim_gb300_build_slices", b._plan.handle, P(c), N, P(cn), B, P(o), P(ws),  # noqa
                                  nbytes, st())
        for _ in range(args.warmup):
            fn()
        t = _time(fn, args.reps, flush)
        out.update(batch=B, atoms=N, slices=S, seconds=t, images_per_s=B / t, slices_per_s=B * S / t)
    elif args.case == "slab":
        from . import atoms as atm
        from . import physics, pot, synth
        d, dz, kev = 0.1, 0.5, 300.0
        el, xyz0 = synth.carbon_slab(0, lateral=n * d, thickness=S * dz)
        mol = atm.centralize(atm.AtomList(el, xyz0))
        ns, _, _ = pot.finalize_slice_size(tuple(mol.space), (d, d), dz, (n, n), None)
        b = backend.MultiSlicesBuilder([6], ns, n, n, dz, d, d)
        wp = backend.WavePropagator(n, n, d, d, kev)
        lam = physics.electron_wave_length_angstrom(kev)
        df, ap = physics.scherzer_condition(lam, 1.0)
        dfs = np.array([df])
        N = int(len(el))
        c = torch.from_numpy(np.ascontiguousarray(mol.coordinates, dtype=np.float32)).to(dev)
        cn = torch.tensor([N], dtype=torch.int32, device=dev)
        o = torch.empty((1, ns, n, n), dtype=torch.float32, device=dev)
        w = torch.empty((1, n, n), dtype=torch.complex64, device=dev)
        img = torch.empty((1, n, n), dtype=torch.float32, device=dev)
        nbytes = int(_native.load().emsim_gb300_build_slices_workspace_size(b._plan.handle, N, 1))
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        build = lambda: _native.call("emsim_gb300_build_slices", b._plan.handle, P(c), N, P(cn), 1, P(o), P(ws),  # noqa
                                     nbytes, st())
        image = lambda: _native.call("emsim_gb300_multislice_image", wp._plan.handle, P(o), ns, ns * n * n, dz,  # noqa
                                     20.0, 1.0, dfs.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), 1, ap, P(img),
                                     P(w), None, 1, st())
        for _ in range(args.warmup):
            build()
            image()
        tb = _time(build, args.reps, flush)
        ti = _time(image, args.reps, flush)
        out.update(atoms=N, slices=ns, build_seconds=tb, image_seconds=ti,
                   build_algo_gbs=(16.0 * N + 4.0 * ns * n * n) / tb / 1e9,
                   per_step_us=1e6 * ti / (ns + 0.5), step_algo_gbs=20.0 * n * n * ns / ti / 1e9)
    elif args.case == "atoms":
        zs = [6, 7, 8, 16]
        b = backend.MultiSlicesBuilder(zs, S, n, n, 2.0, 1.0, 1.0)
        rng = np.random.default_rng(0)
        N = args.atoms * B
        xyz = ((rng.random((N, 3)) * 2 - 1) * np.array([S, n / 2, n / 2]) * 0.9).astype(np.float32)
        per = np.array([args.atoms // 4] * 3 + [args.atoms - 3 * (args.atoms // 4)], dtype=np.uint32)
        counts = np.tile(per, (B, 1))
        c = torch.from_numpy(xyz).to(dev)
        cn = torch.from_numpy(counts.view(np.int32)).to(dev)
        o = torch.empty((B, S, n, n), dtype=torch.float32, device=dev)
        nbytes = int(_native.load().emsim_gb300_build_slices_workspace_size(b._plan.handle, N, B))
        ws = torch.empty(nbytes, dtype=torch.uint8, device=dev)
        fn = lambda: _native.call("emsim_gb300_build_slices", b._plan.handle, P(c), N, P(cn), B, P(o), P(ws),  # noqa
                                  nbytes, st())
        for _ in range(args.warmup):
            fn()
        t = _time(fn, args.reps, flush)
        out.update(batch=B, atoms=N, slices=S, seconds=t, images_per_s=B / t, slices_per_s=B * S / t)
    else:
        zs = [6, 7, 8, 16]
        b = backend.MultiSlicesBuilder(zs, S, n, n, 2.0, 1.0, 1.0)
        rng = np.random.default_rng(0)
        N = args.atoms
        xyz = ((rng.random((N, 3)) * 2 - 1) * np.array([S, n / 2, n / 2])).astype(np.float32)
        cnt = np.array([N // 4, N // 4, N // 4, N - 3 * (N // 4)], dtype=np.int32)
        c = torch.from_numpy(xyz).to(dev)
        cn = torch.from_numpy(cnt).to(dev)
        hist = torch.empty((4, S, n, n), dtype=torch.float32, device=dev)
        fn = lambda: _native.call("emsim_gb300_bin_atoms_multi_slices", b._plan.handle, P(c), N, P(cn),  # noqa
                                  P(hist), st())
        for _ in range(args.warmup):
            fn()
        t = _time(fn, args.reps, flush)
        out.update(atoms=N, slices=S, seconds=t, atoms_per_s=N / t,
                   algo_gbs=(16.0 * N + 4.0 * hist.numel()) / t / 1e9)
    print(json.dumps(out))


if __name__ == "__main__":
    main()
