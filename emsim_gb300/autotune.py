"""Autotuner for the wave passes: picks, per wave size, the row- and column-pass kernels
(TMA-staged persistent or one tile per CTA) and their tile widths by timing a short
multislice on the device, and caches the choice per GPU model and size.

The choice only regroups independent rows or columns, so every setting gives identical
results; only the speed differs.  Cache file: ``$EMSIM_GB300_TUNE_CACHE`` or
``~/.cache/emsim_gb300/autotune.json``.  ``ensure(n1, n2)`` applies a cached choice;
with ``EMSIM_GB300_AUTOTUNE=1`` it also tunes sizes that are not cached yet.
"""
from __future__ import annotations

import ctypes
import json
import os
import threading
from pathlib import Path
from typing import Dict, List, Optional, Tuple

import torch

from . import _native

__all__ = ["get_tuning", "set_tuning", "tune", "ensure", "cache_path"]

_lock = threading.Lock()
_applied: Dict[Tuple[str, int, int], bool] = {}


def cache_path() -> Path:
    p = os.environ.get("EMSIM_GB300_TUNE_CACHE")
    return Path(p) if p else Path.home() / ".cache" / "emsim_gb300" / "autotune.json"


def get_tuning(n: int) -> Dict[str, int]:
    """Current setting for passes of length n and the built-in tiles."""
    out = (ctypes.c_int * 8)()
    _native.call("emsim_gb300_get_pass_tuning", int(n), out)
    v = list(out)
    return {"row_tma": v[0], "row_rows": v[1], "col_tma": v[2], "col_cols": v[3], "default_row_rows_tma": v[4],
            "default_row_rows": v[5], "default_col_cols_tma": v[6], "default_col_cols": v[7]}


def set_tuning(n: int, row_tma: Optional[int] = None, row_rows: int = 0, col_tma: Optional[int] = None,
               col_cols: int = 0) -> None:
    """Set the pass kernels of length n; with neither kernel given, restore the built-in
    setting (the 16-value kernels at 256, 1024, 2048 and 4096, TMA radix-8 elsewhere)."""
    if row_tma is None and col_tma is None:
        _native.call("emsim_gb300_set_pass_tuning", int(n), -2, 0, -1, 0)
        return
    row_tma = -1 if row_tma is None else row_tma
    col_tma = -1 if col_tma is None else col_tma
    _native.call("emsim_gb300_set_pass_tuning", int(n), int(row_tma), int(row_rows), int(col_tma), int(col_cols))


def _gpu_key() -> str:
    return torch.cuda.get_device_name(torch.cuda.current_device())


def _load() -> dict:
    try:
        return json.loads(cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store(data: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(data, indent=1, sort_keys=True))
        tmp.replace(p)
    except OSError:
        pass  # a read-only home still tunes, it only does not remember


def _halvings(default: int, minimum: int) -> List[int]:
    """The built-in tile (0) and up to four halvings of it, down to ``minimum``."""
    out, t = [0], default // 2
    while t >= minimum and len(out) < 5:
        out.append(t)
        t //= 2
    return out


def _time_steps(wp, wave, slices, reps: int) -> float:
    st = torch.cuda.current_stream()
    for _ in range(2):
        wp.multislice_propagate(wave, slices, 2.0)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(st)
    for _ in range(reps):
        wp.multislice_propagate(wave, slices, 2.0)
    b.record(st)
    b.synchronize()
    return a.elapsed_time(b) / reps


def _set_col(n: int, tma: int, cols: int) -> None:
    g = get_tuning(n)
    set_tuning(n, g["row_tma"], g["row_rows"], tma, cols)


def _set_row(n: int, tma: int, rows: int) -> None:
    g = get_tuning(n)
    set_tuning(n, tma, rows, g["col_tma"], g["col_cols"])


def tune(n1: int, n2: int, batch: Optional[int] = None, n_slices: int = 6, reps: int = 5,
         store: bool = True) -> dict:
    """Time the candidate kernels and tiles for an n1 x n2 wave and keep the fastest.

    The column pass (length n1) is tuned first, then the row pass (length n2).  Returns
    {"row": [tma, rows], "col": [tma, cols], "ms": time of one multislice call}; the
    choice is applied and, with ``store``, cached."""
    from .backend import WavePropagator
    dev = torch.device("cuda", torch.cuda.current_device())
    if batch is None:
        batch = max(1, (32 * 256 * 256) // (n1 * n2))
    g = torch.Generator(device=dev)
    g.manual_seed(1)
    wave = torch.randn((batch, n1, n2), dtype=torch.complex64, device=dev, generator=g)
    slices = torch.rand((n_slices, n1, n2), dtype=torch.float32, device=dev, generator=g) * 50
    slices = slices.unsqueeze(0).expand(batch, -1, -1, -1).contiguous()
    wp = WavePropagator(n1, n2, 1.0, 1.0, 200.0)
    g1, g2 = get_tuning(n1), get_tuning(n2)
    best_t = float("inf")
    best_col = (g1["col_tma"], g1["col_cols"])
    # column kernels: TMA radix-8 (-1), plain radix-8 (0) and, at lengths 256..4096, TMA
    # with 16 values per thread (2, 512 threads: 512 / (n1 / 16) columns per tile by default)
    col_kernels = {-1: (g1["default_col_cols_tma"], 2), 0: (g1["default_col_cols"], 1)}
    if 256 <= n1 <= 4096:
        col_kernels[2] = (max(2, 512 // (n1 // 16)), 2)
    for tma, (default_cols, min_cols) in col_kernels.items():
        for cols in _halvings(default_cols, min_cols):
            _set_col(n1, tma, cols)
            t = _time_steps(wp, wave, slices, reps)
            if t < best_t:
                best_col, best_t = (tma, cols), t
    _set_col(n1, *best_col)
    best_row = (g2["row_tma"], g2["row_rows"])
    # row kernels: TMA radix-8 (-1), plain radix-8 (0) and, at lengths 256..4096, TMA with 16
    # values per thread (2, 256 threads: 256 / (n2 / 16) rows per tile by default)
    row_kernels = {-1: g2["default_row_rows_tma"], 0: g2["default_row_rows"]}
    if 256 <= n2 <= 4096:
        row_kernels[2] = max(1, 256 // (n2 // 16))
    for tma, default_rows in row_kernels.items():
        for rows in _halvings(default_rows, 1):
            _set_row(n2, tma, rows)
            t = _time_steps(wp, wave, slices, reps)
            if t < best_t:
                best_row, best_t = (tma, rows), t
    _set_row(n2, *best_row)
    result = {"row": list(best_row), "col": list(best_col), "ms": best_t, "batch": batch, "n_slices": n_slices}
    with _lock:
        if store:
            data = _load()
            data.setdefault(_gpu_key(), {})[f"{n1}x{n2}"] = result
            _store(data)
        _applied[(_gpu_key(), n1, n2)] = True
    return result


def ensure(n1: int, n2: int) -> Optional[dict]:
    """Apply the cached choice for an n1 x n2 wave (tuning it first when
    EMSIM_GB300_AUTOTUNE=1 and nothing is cached).  Returns the choice or None."""
    key = (_gpu_key(), int(n1), int(n2))
    if _applied.get(key):
        return None
    entry = _load().get(key[0], {}).get(f"{n1}x{n2}")
    if entry is None:
        if os.environ.get("EMSIM_GB300_AUTOTUNE") == "1":
            return tune(n1, n2)
        _applied[key] = True
        return None
    _set_col(int(n1), *entry["col"])
    _set_row(int(n2), *entry["row"])
    _applied[key] = True
    return entry
