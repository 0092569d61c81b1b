"""The pass autotuner: every kernel / tile choice gives bitwise-identical waves, tuning
picks a valid choice, and the cache round-trips."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def eng():
    import emsim_gb300.build as b
    b.build()
    import torch

    from emsim_gb300 import autotune, backend
    return torch, autotune, backend


@pytest.mark.parametrize("n1,n2", [(256, 256), (128, 512), (512, 64)])
def test_every_setting_gives_identical_waves(eng, n1, n2):
    torch, autotune, backend = eng
    rng = np.random.default_rng(n1 + n2)
    w = (rng.normal(size=(3, n1, n2)) + 1j * rng.normal(size=(3, n1, n2))).astype(np.complex64)
    s = (rng.random((4, n1, n2)) * 30).astype(np.float32)
    wp = backend.WavePropagator(n1, n2, 0.7, 0.7, 200.0)
    g1, g2 = autotune.get_tuning(n1), autotune.get_tuning(n2)
    try:
        # the radix-8 family (TMA and one-tile-per-CTA kernels, any tile) against itself
        autotune.set_tuning(n1, -1, 0, -1, 0)
        autotune.set_tuning(n2, -1, 0, -1, 0)
        ref = np.asarray(wp.multislice_propagate(w, s, 2.0).get())
        for ct, cc in [(-1, g1["default_col_cols_tma"] // 2), (0, 0), (0, max(1, g1["default_col_cols"] // 4))]:
            for rt, rr in [(-1, max(1, g2["default_row_rows_tma"] // 2)), (0, 0), (0, max(1, g2["default_row_rows"] // 2))]:
                autotune._set_col(n1, ct, cc)
                autotune._set_row(n2, rt, rr)
                got = np.asarray(wp.multislice_propagate(w, s, 2.0).get())
                np.testing.assert_array_equal(got, ref)
    finally:
        autotune.set_tuning(n1)
        autotune.set_tuning(n2)


@pytest.mark.parametrize("n1,n2", [(256, 256), (256, 512), (512, 256), (64, 256)])
def test_radix16_settings(eng, n1, n2):
    """The radix-16 kernels of length 256 (row and column passes): every tile choice gives
    bitwise-identical waves, within 1e-5 (relative L2) of the radix-8 kernels."""
    torch, autotune, backend = eng
    rng = np.random.default_rng(n1 * 3 + n2)
    w = (rng.normal(size=(2, n1, n2)) + 1j * rng.normal(size=(2, n1, n2))).astype(np.complex64)
    s = (rng.random((4, n1, n2)) * 30).astype(np.float32)
    wp = backend.WavePropagator(n1, n2, 0.7, 0.7, 200.0)
    try:
        autotune.set_tuning(256, -1, 0, -1, 0)
        ref8 = np.asarray(wp.multislice_propagate(w, s, 2.0).get())
        ref16 = None
        for rows, cols in [(0, 0), (8, 16), (4, 8), (2, 4), (1, 2)]:
            autotune.set_tuning(256, 2, rows, 2, cols)
            got = np.asarray(wp.multislice_propagate(w, s, 2.0).get())
            if ref16 is None:
                ref16 = got
                err = np.linalg.norm(got - ref8) / np.linalg.norm(ref8)
                assert 0 <= err < 1e-5, err
            np.testing.assert_array_equal(got, ref16)
    finally:
        autotune.set_tuning(256)


def test_tune_and_cache(eng, tmp_path, monkeypatch):
    torch, autotune, backend = eng
    monkeypatch.setenv("EMSIM_GB300_TUNE_CACHE", str(tmp_path / "tune.json"))
    try:
        res = autotune.tune(256, 256, batch=8, n_slices=3, reps=2)
        assert res["col"][0] in (-1, 0, 2) and res["row"][0] in (-1, 0, 2) and res["ms"] > 0
        data = autotune._load()
        assert any("256x256" in v for v in data.values())
        autotune.set_tuning(256)
        autotune._applied.clear()
        entry = autotune.ensure(256, 256)
        g = autotune.get_tuning(256)
        assert [g["col_tma"], g["col_cols"]] == [(-1 if entry["col"][0] == 1 else entry["col"][0]), entry["col"][1]]
    finally:
        autotune.set_tuning(256)
        autotune._applied.clear()
