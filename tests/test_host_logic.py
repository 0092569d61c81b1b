"""Host-side logic of the product package, on CPU: front-end geometry, physics and
scattering factors against the reference goldens, the algebra behind the fused slice
build, backend registration and the C ABI's exported symbols."""
import ctypes
import re
import types
from pathlib import Path

import numpy as np
import pytest

from emsim_gb300 import _native, atoms, config, elem, physics
from oracle import multislice as om

ROOT = Path(__file__).resolve().parent.parent


def test_physics_matches_golden(golden):
    g = golden("physics")
    np.testing.assert_array_equal([physics.electron_wave_length_angstrom(k) for k in g["kev"]], g["wave_length"])
    np.testing.assert_array_equal([physics.electron_relativity_gamma(k) for k in g["kev"]], g["gamma"])
    np.testing.assert_array_equal([physics.interaction_parameter(k) for k in g["kev"]], g["sigma"])
    for kev, cs, df, ap in g["scherzer"]:
        assert physics.scherzer_condition(physics.electron_wave_length_angstrom(kev), cs) == (df, ap)


@pytest.mark.parametrize("tag", ["a", "b", "c"])
def test_scattering_factors_match_golden(golden, tag):
    g = golden("scattering")
    n1, n2, d1, d2 = g[f"grid_{tag}"]
    np.testing.assert_array_equal(elem.scattering_factors2d(list(g["zs"]), int(n1), int(n2), d1, d2),
                                  g[f"sf2d_{tag}"])
    np.testing.assert_array_equal(elem.scattering_factors_half(list(g["zs"]), int(n1), int(n2), d1, d2),
                                  g[f"half_{tag}"])


def test_front_end_geometry_matches_oracle(golden):
    g = golden("pipe")
    mol = atoms.AtomList(g["blob_elements"], g["blob_coords"])
    c = atoms.centralize(mol)
    np.testing.assert_array_equal(c.coordinates, om.centralize(g["blob_coords"]))
    s, uz, cnt = atoms.sort_elements_and_count(c, [1, 8])
    _, xyz, uz2, cnt2 = om.sort_elements_and_count(g["blob_elements"], c.coordinates, [1, 8])
    np.testing.assert_array_equal(uz, uz2)
    np.testing.assert_array_equal(cnt, cnt2)
    assert 1 in uz and cnt[list(uz).index(1)] == 0
    assert atoms.determine_box_size(tuple(s.space), (2.0, 1.0, 1.0), (None, 32, 32)) == \
        om.finalize_slice_size(s.space, (1.0, 1.0), 2.0, 32, None)
    # flat axes become 3 A thick
    assert atoms.determine_box_size((0.0, 10.0, 10.0), (2.0, 1.0, 1.0), (None, None, None)) == (2, 10, 10)


def test_rotation_matches_reference_convention():
    q = np.array([0.5, 0.5, 0.5, 0.5])
    np.testing.assert_allclose(atoms.get_rotation_mattrices(q)[0], om.rotation_matrix(q))
    r = atoms.get_rotation_mattrices(atoms.random_uniform_quaternions(5, np.random.default_rng(0)))
    np.testing.assert_allclose(r @ r.transpose(0, 2, 1), np.broadcast_to(np.eye(3), (5, 3, 3)), atol=1e-12)


def _bandlimit_full(n1, n2):
    """Python restatement of the engine's full-spectrum band-limit (slices.cu)."""
    r = min(n1, n2) // 2

    def centred(i, n):
        return ((i + n // 2) % n) + (-n // 2)

    h2 = n2 // 2

    def G(i, j):
        if j > h2:
            return 0.0
        fil = 1.0 if centred(i, n1) ** 2 + centred(j, n2) ** 2 <= r * r else 0.0
        selfc = j == 0 or (n2 % 2 == 0 and j == h2)
        return (1.0 if selfc else 2.0) * fil

    F = np.empty((n1, n2))
    for i in range(n1):
        for j in range(n2):
            F[i, j] = 0.5 * (G(i, j) + G((n1 - i) % n1, (n2 - j) % n2))
    return F


@pytest.mark.parametrize("n1,n2", [(16, 16), (15, 15), (12, 20), (9, 14)])
def test_bandlimit_as_full_spectrum_filter(n1, n2):
    """irfft2(rfft2(V) * fil_half) == Re ifft2(F * fft2(V)) with the symmetrised F, also
    for odd sizes where numpy's centred grid makes fil asymmetric."""
    rng = np.random.default_rng(n1 * 100 + n2)
    v = rng.normal(size=(n1, n2))
    ref = np.fft.irfft2(np.fft.rfft2(v) * om.bandlimit_mask_half(n1, n2), s=(n1, n2))
    F = _bandlimit_full(n1, n2)
    np.testing.assert_array_equal(F, F[(-np.arange(n1)) % n1][:, (-np.arange(n2)) % n2])
    got = np.fft.ifft2(F * np.fft.fft2(v))
    assert np.abs(got.imag).max() < 1e-12
    np.testing.assert_allclose(got.real, ref, atol=1e-12)


def test_packed_pair_slice_build():
    """V_a + i V_b = ifft2(sum_e T_e fft2(h_ea + i h_eb)) for real symmetric T_e: two
    slices per complex transform, as the engine builds them."""
    rng = np.random.default_rng(5)
    n1 = n2 = 16
    sf = om.scattering_factors_half([6, 8], n1, n2, 0.5, 0.5)
    hist = rng.poisson(0.3, size=(2, 2, n1, n2)).astype(np.float64)
    ref = om.make_slices(hist, sf, "fftw", np.float64)
    F = _bandlimit_full(n1, n2)
    h = n2 // 2 + 1
    full = np.empty((2, n1, n2))
    for e in range(2):
        for i in range(n1):
            for j in range(n2):
                full[e, i, j] = sf[e, i, j] if j < h else sf[e, (n1 - i) % n1, n2 - j]
    T = F[None] * full / (n1 * n2)
    z = hist[:, 0] + 1j * hist[:, 1]
    w = np.fft.ifft2((T * np.fft.fft2(z)).sum(axis=0)) * (n1 * n2)
    np.testing.assert_allclose(np.maximum(w.real, 1e-13), ref[0], atol=1e-12)
    np.testing.assert_allclose(np.maximum(w.imag, 1e-13), ref[1], atol=1e-12)


def test_register_with_emsim_config():
    calls = []
    cfg = types.SimpleNamespace(_current_backend="numpy-backend", set_backend=lambda b="numpy": calls.append(b))
    fake = types.SimpleNamespace(config=cfg)
    config.register(fake)
    config.register(fake)  # idempotent
    cfg.set_backend("gb300")
    assert isinstance(cfg._current_backend, config.Gb300Backend)
    cfg.set_backend("fftw")
    assert calls == ["fftw"]


# ---------------------------------------------------------------------------------
# C ABI
# ---------------------------------------------------------------------------------
def _declared_symbols():
    text = (ROOT / "include" / "emsim_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(emsim_gb300_[a-z0-9_]+)\s*\(", text)))


def test_capi_exports_every_declared_symbol():
    lib = _native.load()
    declared = _declared_symbols()
    assert len(declared) >= 15
    for name in declared:
        assert hasattr(lib, name), name
        assert name in _native.SIGNATURES, f"{name} missing from the ctypes signatures"
    assert set(_native.SIGNATURES) == set(declared)
    assert lib.emsim_gb300_abi_version() == 1


def test_capi_rejects_bad_arguments_without_gpu():
    lib = _native.load()
    h = ctypes.c_void_p()
    assert lib.emsim_gb300_wave_plan_create(0, 8, 1.0, 1.0, 0.025, 1.4, ctypes.byref(h)) == 1
    assert "positive" in _native.last_error()
    assert lib.emsim_gb300_wave_plan_create(8, 8, -1.0, 1.0, 0.025, 1.4, ctypes.byref(h)) == 1
    assert lib.emsim_gb300_slice_plan_create(None, 1, 1, 8, 8, 1.0, 1.0, 1.0, 1, ctypes.byref(h)) == 1
    assert lib.emsim_gb300_intensity(None, None, 4, None) == 1
    assert lib.emsim_gb300_make_slices_workspace_size(None) == 0
    with pytest.raises(_native.NativeError):
        _native.call("emsim_gb300_init_wave", None, 1.0, None, 1, None)


def test_native_missing_library_fails_loudly(tmp_path):
    with pytest.raises(_native.NativeUnavailable):
        _native.load(tmp_path / "nope.so")


def test_philox_known_answers_and_water_model():
    """Philox4x32-10 restatement against the published known-answer vectors (Random123),
    the vectorised form against the scalar one, and the Poisson inversion's mean."""
    import numpy as np

    from oracle import water
    kat = [((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
           ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
           ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
            (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1))]
    for c, k, want in kat:
        assert water.philox4x32_10(c, k) == list(want)
    v = np.array([0, 1, 7, 2 ** 33 + 5, 123456789012], dtype=np.uint64)
    seed, stream = 0x0123456789ABCDEF, 3
    w0, w1 = water.philox_vec(v, stream, seed)
    for i, x in enumerate(v):
        ref = water.philox4x32_10((int(x) & 0xFFFFFFFF, int(x) >> 32, stream, 0), (seed & 0xFFFFFFFF, seed >> 32))
        assert (int(w0[i]), int(w1[i])) == (ref[0], ref[1])
    words, _ = water.philox_vec(np.arange(200_000, dtype=np.uint64), 0, 99)
    for lam in (0.062, 0.5, 3.0):
        k = water.poisson_inv(words, lam)
        assert abs(k.mean() - lam) < 5 * np.sqrt(lam / len(k))


def test_pass_tuning_table_host_side():
    """emsim_gb300_set/get_pass_tuning validate and store without touching a GPU."""
    import ctypes

    from emsim_gb300 import _native
    lib = _native.load()
    out = (ctypes.c_int * 8)()
    assert lib.emsim_gb300_get_pass_tuning(256, out) == 0
    assert list(out)[:4] == [2, 4, 2, 8]  # built-in: the 16-value kernels, 4 rows and 8 columns per tile
    assert list(out)[4:] == [8, 8, 16, 16]  # built-in tiles at 256: 256 threads / 32 per row, 512 / 32 columns
    for n, want in [(512, [-1, 0, -1, 0]), (1024, [2, 0, 2, 0]), (2048, [2, 1, 2, 0]), (4096, [2, 0, 2, 0]),
                    (64, [-1, 0, -1, 0])]:
        lib.emsim_gb300_get_pass_tuning(n, out)
        assert list(out)[:4] == want, n
    assert lib.emsim_gb300_set_pass_tuning(256, 0, 4, 1, 8) == 0
    lib.emsim_gb300_get_pass_tuning(256, out)
    assert list(out)[:4] == [0, 4, -1, 8]
    assert lib.emsim_gb300_set_pass_tuning(256, -1, 0, -1, 0) == 0
    assert lib.emsim_gb300_set_pass_tuning(100, -1, 0, -1, 0) == 1  # not a power of two
    assert lib.emsim_gb300_set_pass_tuning(256, 3, 0, -1, 0) == 1  # row kernels: -1, 0, 1, 2 (radix 16)
    assert lib.emsim_gb300_set_pass_tuning(256, -1, 0, 3, 0) == 1  # column kernels: -1, 0, 1, 2 (radix 16)
    assert lib.emsim_gb300_set_pass_tuning(256, 2, 4, -1, 0) == 0
    lib.emsim_gb300_get_pass_tuning(256, out)
    assert list(out)[:2] == [2, 4]
    assert lib.emsim_gb300_set_pass_tuning(256, -1, -3, -1, 0) == 1
    assert lib.emsim_gb300_set_pass_tuning(256, -2, 0, 0, 0) == 0  # back to the built-in setting
    lib.emsim_gb300_get_pass_tuning(256, out)
    assert list(out)[:4] == [2, 4, 2, 8]


def test_synthetic_blob_matches_oracle_generator():
    """The package's seeded blob generator (used by the benchmark) reproduces the one the
    tests use, so benchmark inputs and parity inputs are the same atoms."""
    import numpy as np

    from emsim_gb300 import synth
    from oracle import multislice as om
    a, b = synth.protein_blob(3000, 15.0, 9), om.protein_blob(3000, 15.0, 9)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    mix = synth.batching_mix(4, seed=2)
    assert len(mix) == 4 and {r for _, _, r in mix} <= {256, 512}
    assert all(set(np.unique(el)) <= {1, 6, 7, 8, 16} for el, _, _ in mix)
    assert np.any(mix[1][0] == 1) and not np.any(mix[0][0] == 1)  # odd blobs carry ice


def test_pending_images_reassemble_input_order():
    """PendingImages (Pipe.submit_batch's handle) waits on its event once, returns the
    images of its groups in input order as views of the page-locked buffers, and reports
    done() from the event; a completed handle never waits.  Host logic, with a fake
    event and CPU tensors standing in for the page-locked copies."""
    import torch

    from emsim_gb300.pipe import PendingImages

    class FakeEvent:
        def __init__(self):
            self.waits = 0
            self.ready = False

        def query(self):
            return self.ready

        def synchronize(self):
            self.waits += 1
            self.ready = True

    a = torch.arange(3 * 2 * 2, dtype=torch.float32).reshape(3, 2, 2)
    b = 100 + torch.arange(2 * 4 * 4, dtype=torch.float32).reshape(2, 4, 4)
    ev = FakeEvent()
    p = PendingImages(5, [([4, 0, 2], a, None), ([1, 3], b, None)], ev)
    assert not p.done()
    out = p.result()
    assert ev.waits == 1 and p.done()
    assert [o.shape for o in out] == [(2, 2), (4, 4), (2, 2), (4, 4), (2, 2)]
    np.testing.assert_array_equal(out[4], a[0].numpy())
    np.testing.assert_array_equal(out[0], a[1].numpy())
    np.testing.assert_array_equal(out[2], a[2].numpy())
    np.testing.assert_array_equal(out[1], b[0].numpy())
    np.testing.assert_array_equal(out[3], b[1].numpy())
    assert np.shares_memory(out[0], a.numpy())  # views of the buffer, no copy
    assert p.result() is out and ev.waits == 1
    done = PendingImages.completed([np.zeros(2)])
    assert done.done() and len(done.result()) == 1


def test_emsim_results_in_input_order_one_at_a_time_and_batched():
    """EMSim (emsim/simulator.py:21-91) hands every image to the handler in input order
    with its label, logs and skips a failing molecule; with batch_size > 1 it submits
    groups through submit_batch, two in flight, and a group that fails as a whole (at
    submission or when collected) is rerun molecule by molecule.  A fake pipe stands in
    for the GPU."""
    from emsim_gb300.simulator import EMSim

    class Mol:
        def __init__(self, k, bad=False, late=False):
            self.label, self.k, self.bad, self.late = f"m{k}", k, bad, late

    class FakePending:
        def __init__(self, imgs, fail):
            self.imgs, self.fail = imgs, fail

        def result(self):
            if self.fail:
                raise RuntimeError("device error reported at collection")
            return self.imgs

    class FakePipe:
        def __init__(self):
            self.groups, self.single = [], []

        def run(self, mol):
            self.single.append(mol.k)
            if mol.bad:
                raise ValueError("bad molecule")
            return np.full(3, mol.k, np.float32)

        def submit_batch(self, mols):
            self.groups.append([m.k for m in mols])
            if any(m.bad for m in mols):
                raise ValueError("a bad molecule in the group")
            return FakePending([np.full(3, m.k, np.float32) for m in mols], any(m.late for m in mols))

    mols = [Mol(k, bad=(k == 5), late=(k == 9)) for k in range(11)]
    want = [f"m{k}" for k in range(11) if k != 5]
    for bs in (1, 4):
        got = []
        fake = FakePipe()
        EMSim(fake, mols, lambda img, label: got.append((label, img.copy())), batch_size=bs).run()
        assert [lab for lab, _ in got] == want
        assert all(img[0] == int(lab[1:]) for lab, img in got)
        if bs == 1:
            assert fake.groups == [] and fake.single == list(range(11))
        else:
            assert fake.groups == [[0, 1, 2, 3], [4, 5, 6, 7], [8, 9, 10]]
            assert fake.single == [4, 5, 6, 7, 8, 9, 10]  # the two failed groups, rerun one by one
    with pytest.raises(ValueError):
        EMSim(FakePipe(), mols, lambda *a: None, batch_size=0)


def test_wait_limit_setting_host_side():
    """emsim_gb300_set/get_wait_limit_ns store the bounded-wait limit without a GPU and
    refuse limits below 1 ms (a pipelined kernel would give up on copies still landing)."""
    lib = _native.load()
    default = lib.emsim_gb300_get_wait_limit_ns()
    assert default == 2_000_000_000
    assert lib.emsim_gb300_set_wait_limit_ns(999_999) == 1
    assert "1 ms" in _native.last_error()
    assert lib.emsim_gb300_get_wait_limit_ns() == default
    assert lib.emsim_gb300_set_wait_limit_ns(50_000_000) == 0
    assert lib.emsim_gb300_get_wait_limit_ns() == 50_000_000
    assert lib.emsim_gb300_set_wait_limit_ns(default) == 0
    assert lib.emsim_gb300_wait_timeout_probe(10, None, None) == 1  # null output, limit below 1 us


def test_frontend_trace_binds_to_backend_signatures():
    """Every backend call that emsim's own front-end made (recorded from the reference
    package: five atoms through pot.build_one_slice / TEM.get_wave_propagator /
    init_wave / slice_transmit / lens_propagate, and Pipe.run of a blob) binds to the
    GB300 backend's constructors and methods with the same arguments."""
    import inspect

    import frontend_trace
    from emsim_gb300 import backend

    trace, arrays = frontend_trace.load()
    records = trace["records"]
    assert {r["cls"] for r in records} == {"OneSliceBuilder", "MultiSlicesBuilder", "WavePropagator"}
    assert {r["method"] for r in records if r["op"] == "call"} >= {
        "bin_atoms_one_slice", "make_one_slice", "bin_atoms_multi_slices", "make_multi_slices", "init_wave",
        "slice_transmit", "multislice_propagate", "lens_propagate"}
    placeholder = object()
    for r in records:
        cls = getattr(backend, r["cls"])
        fn = cls.__init__ if r["op"] == "new" else getattr(cls, r["method"])
        args = [placeholder] + [placeholder] * len(r["args"])  # self + positional arguments
        inspect.signature(fn).bind(*args, **{k: placeholder for k in r["kwargs"]})


def test_register_with_the_reference_emsim_config():
    """config.register on the reference's own emsim.config module (where its source tree
    is given by EMSIM_REFERENCE_ROOT): set_backend("gb300") makes emsim's front-end
    resolve the GB300 classes, and the reference's own names keep working."""
    from oracle import ref_numpy
    if not ref_numpy.available():
        pytest.skip("reference source tree not available (EMSIM_REFERENCE_ROOT)")
    from emsim_gb300 import backend
    em = ref_numpy.load()
    config.register(em)
    try:
        em.config.set_backend("gb300")
        cur = em.config.get_current_backend()
        assert cur.one_slice_builder is backend.OneSliceBuilder
        assert cur.multi_slices_builder is backend.MultiSlicesBuilder
        assert cur.wave_propagator is backend.WavePropagator
        # the front-end resolves the class at call time (wave.py:7-16)
        calls = []
        orig = backend.WavePropagator.__init__

        def spy(self, *a, **k):
            calls.append(a)
            orig(self, *a, **k)

        backend.WavePropagator.__init__ = spy
        try:
            with pytest.raises(Exception):  # no GPU here: the plan creation itself fails
                em.wave.get_raw_wave_propagator(64, 0.5, 200.0)
        finally:
            backend.WavePropagator.__init__ = orig
        assert calls == [(64, 64, 0.5, 0.5, 200.0)]
    finally:
        em.config.set_backend("numpy")
    assert em.config.get_current_backend().wave_propagator.__module__.endswith("wave_propagator_numpy")


def test_pipe_graph_cache_sightings_lru_and_drop():
    from emsim_gb300.pipe import _GraphCache
    c = _GraphCache(max_entries=2)
    assert c.sighting("a", 1) == 1 and c.sighting("a", 1) == 2 and c.sighting("b", 1) == 1
    c.put("a", 1, "g1")
    c.put("a", 2, "g2")
    assert c.get("a", 1) == "g1"  # now the most recently used
    c.put("a", 3, "g3")           # drops key 2, the least recently used
    assert c.get("a", 2) is None and c.get("a", 1) == "g1" and c.get("a", 3) == "g3"
    assert c.get("b", 1) is None and len(c) == 2
    c.drop("a")                   # the buffer set grew: its graphs and sightings go
    assert len(c) == 0 and c.sighting("a", 1) == 1 and c.sighting("b", 1) == 2
