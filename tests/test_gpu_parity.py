"""Parity of the CUDA engine with the reference, through the C ABI.

The oracle for positions and times is the reference's own hot-path source compiled by nvcc for the GPU
(oracle/ref_device.cu; fixtures tests/golden/dev_*.npz written on a GB300 by tests/golden/make_device_golden.py):

* Arithmetic (the strict gate).  Built without multiply-add contraction (nvcc --fmad=false) on both sides, every
  binary32 operation is rounded on its own, so results depend only on the operations the source performs and on
  CUDA's math functions, which both call.  The engine so built must reproduce the reference so built bit for bit:
  at least 99.9 % of photons with identical records and flag histories, on every fixture and in every kernel form.
* Production build.  With contraction on (the default of both builds) the compiler fuses mul+add pairs per kernel,
  and the reference's own source built with and without contraction already disagrees beyond 1e-3 mm on long or
  mirrored paths (the fixture records that fraction).  The engine's production build must reproduce at least 99.9 %
  of flag histories and integer words, and have positions within 1e-3 mm (one ulp where larger) and times within
  1e-3 ns for at least 99.9 % of photons, or for at least as many photons as those two builds of the reference
  agree on, whichever is smaller.

Integer work (RNG stream, hit selection and order) is bit-exact.
"""
import numpy as np
import pytest

from conftest import SIM_FIXTURES, assert_photons_agree, golden_arrays, load_golden

pytestmark = pytest.mark.gpu

POS_TOL_MM = 1e-3
TIME_TOL_NS = 1e-3


@pytest.fixture(scope="module")
def E():
    import __graft_entry__ as ge
    ge.build()
    from eic_opticks_gb300 import engine
    return engine


def test_rng_sequence_bit_exact(E, oracle):
    z = load_golden("philox.npz")
    for case, want in zip(z["cases"], z["uniforms"]):
        seed, sub, off, skip = (int(x) for x in case)
        got = E.rng_sequence(seed, sub, off + skip, 1, want.shape[0])[0]
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), case
    got = E.rng_sequence(0, 1000, 300000, 256, 40)
    for i in (0, 17, 255):
        want = oracle.philox_uniforms(0, 1000 + i, 0, 300000, 40)
        assert np.array_equal(got[i].view(np.uint32), want.view(np.uint32))


def test_texture_filter_matches_emulation(E, oracle):
    from eic_opticks_gb300 import geometry as G
    arrays = G.water_cube().arrays()
    eng = E.Engine(arrays)
    rng = np.random.default_rng(3)
    bnd = arrays["bnd"].reshape(-1, arrays["bnd"].shape[-2], 4)
    xy = np.stack([rng.uniform(-0.1, 1.1, 20000), rng.uniform(0, 1, 20000)], axis=1).astype(np.float32)
    # boundary lookups as qbnd::boundary_lookup makes them: wavelength on the domain, y at row centres
    nm = rng.uniform(60, 820, 20000).astype(np.float32)
    rows = rng.integers(0, bnd.shape[0], 20000)
    xb = ((((nm - np.float32(60.0)) / np.float32(1.0)) + np.float32(0.5)) / np.float32(761.0)).astype(np.float32)
    yb = ((rows.astype(np.float32) + np.float32(0.5)) / np.float32(bnd.shape[0])).astype(np.float32)
    xy_b = np.stack([xb, yb], axis=1)
    hw = eng.texture_lookup(0, xy_b)
    emu = oracle.tex_lookup(bnd, xy_b)
    exact = np.all(hw.view(np.uint32) == emu.view(np.uint32), axis=1).mean()
    print("boundary texture: bit-exact fraction %.6f" % exact)
    assert exact == 1.0
    # ICDF as qscint samples it: any x (wrap included) on the three row centres
    rows_y = np.array([0.5 / 3.0, 1.5 / 3.0, 2.5 / 3.0], dtype=np.float32)
    xy_c = np.stack([xy[:, 0], rows_y[rng.integers(0, 3, len(xy))]], axis=1)
    hw1 = eng.texture_lookup(1, xy_c)
    emu1 = oracle.tex_lookup(arrays["icdf"], xy_c)
    exact1 = (hw1.view(np.uint32) == emu1.view(np.uint32)).mean()
    print("icdf texture (row centres): bit-exact fraction %.6f" % exact1)
    assert exact1 == 1.0
    # both weights fractional (never sampled by the photon path): within one 1/256 weight step of the row spread
    hw2 = eng.texture_lookup(1, xy)
    emu2 = oracle.tex_lookup(arrays["icdf"], xy)
    icdf = arrays["icdf"]
    spread = icdf.max() - icdf.min()
    err = np.abs(hw2 - emu2)
    print("icdf texture (bilinear): bit-exact %.4f max err %.3g (row spread / 256 = %.3g)"
          % ((hw2 == emu2).mean(), err.max(), spread / 256))
    assert err.max() <= spread / 256 * 1.01
    u = rng.uniform(0, 1, 50000).astype(np.float32)
    w = eng.scint_wavelength(u)
    assert np.all((w > 60) & (w < 900))
    eng.close()


@pytest.mark.parametrize("name", SIM_FIXTURES)
def test_flag_history_matches_reference_host_build(E, name):
    """The reference's headers compiled for the host (no contraction, libm) wrote these fixtures: the engine
    reproduces their flag histories, flags and hit decisions.  Positions and times are held to the device builds
    above (libm and CUDA's logf/sincosf differ in the last bits)."""
    z = load_golden("sim_%s.npz" % name)
    arrays = golden_arrays(z)
    eng = E.Engine(arrays, record_photon=1, record_seq=1)
    inp = z["input_photon"] if len(z["input_photon"]) else None
    eng.simulate(int(z["event_index"]), z["gs"], inp)
    p, s = eng.photons(), eng.seq()
    eng.close()
    ref, rseq = z["photon"], z["seq"]
    assert len(p) == len(ref)
    same = np.all(s["seqhis"] == rseq["seqhis"], axis=1)
    flags = (p["flagmask"] == ref["flagmask"]) & (p["orient_boundary_flag"] == ref["orient_boundary_flag"])
    print("%s: %d photons, history match %.5f, flags match %.5f" % (name, len(p), same.mean(), flags.mean()))
    assert same.mean() >= 0.999 and flags.mean() >= 0.999


def strict_compare(eng_p, eng_seqhis, ref_p, ref_seqhis):
    """The parity bars against the reference's own device arithmetic: flag history (seqhis) identical; for those
    photons, positions within 1e-3 mm and times within 1e-3 ns, or one ulp of the value where that is larger;
    integer words (flags, boundary, identity, index, instance) identical."""
    same = np.all(eng_seqhis == ref_seqhis, axis=1)
    a, b = eng_p[same], ref_p[same]
    pos_ok = np.all(np.abs(a["pos"] - b["pos"]) <= np.maximum(POS_TOL_MM, np.spacing(np.abs(b["pos"]))), axis=1)
    t_ok = np.abs(a["time"] - b["time"]) <= np.maximum(TIME_TOL_NS, np.spacing(np.abs(b["time"])))
    wa, wb = a.view(np.uint32).reshape(-1, 16), b.view(np.uint32).reshape(-1, 16)
    int_ok = np.all(wa[:, [7, 12, 13, 14, 15]] == wb[:, [7, 12, 13, 14, 15]], axis=1)
    exact = np.all(wa == wb, axis=1)
    n = max(1, len(same))
    m = max(1, int(same.sum()))
    return {"photons": len(same), "history": same.sum() / n, "pos": pos_ok.sum() / m, "time": t_ok.sum() / m,
            "ints": int_ok.sum() / m, "bit_exact": exact.sum() / n}


def _mdg():
    import importlib.util
    import os
    from conftest import GOLDEN
    spec = importlib.util.spec_from_file_location("make_device_golden", os.path.join(GOLDEN, "make_device_golden.py"))
    mdg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mdg)
    return mdg


CONFIGS = ["cfg1_nested_boxes", "cfg2_crystal_array", "cfg3_water_cube", "cfg5_large_sphere"]


def _device_golden(name, variant=""):
    import os
    from conftest import GOLDEN
    path = os.path.join(GOLDEN, "dev_%s%s.npz" % (variant + "_" if variant else "", name))
    if not os.path.exists(path):
        pytest.fail("reference-device fixture %s missing" % path)
    return np.load(path, allow_pickle=False)


def _assert_production(name, r, d):
    """The production-build bars (module docstring): the strict fraction, or the reference's own agreement between
    its builds with and without contraction where that is lower."""
    pos_bar = min(0.999, float(d["self_pos"]))
    time_bar = min(0.999, float(d["self_time"]))
    print("%s vs reference device build: %s | reference with vs without contraction: within 1e-3 mm %.5f, "
          "1e-3 ns %.5f" % (name, " ".join("%s %.6g" % kv for kv in r.items()), d["self_pos"], d["self_time"]))
    assert r["history"] >= 0.999 and r["ints"] >= 0.999
    assert r["pos"] >= pos_bar and r["time"] >= time_bar


@pytest.mark.parametrize("name", SIM_FIXTURES)
def test_simulate_matches_reference_device(E, name):
    """Every host fixture's inputs against the reference's headers compiled by nvcc and run on the GPU."""
    z = load_golden("sim_%s.npz" % name)
    d = _device_golden(name)
    eng = E.Engine(golden_arrays(z), record_photon=1, record_seq=1)
    inp = z["input_photon"] if len(z["input_photon"]) else None
    eng.simulate(int(z["event_index"]), z["gs"], inp)
    r = strict_compare(eng.photons(), eng.seq()["seqhis"], d["photon"], d["seq"]["seqhis"])
    eng.close()
    _assert_production(name, r, d)


@pytest.mark.parametrize("name", CONFIGS)
def test_benchmark_configs_match_reference_device(E, name):
    """100k-photon samples of the benchmark configurations (the full 20,000-sensor geometry for the large sphere)
    against the reference's headers compiled by nvcc and run on the GPU."""
    mdg = _mdg()
    d = _device_golden(name)
    arrays, gs, inp, ev = mdg.config_inputs(name)
    assert mdg.geometry_digest(arrays) == str(d["geometry_sha256"]), "geometry generator changed since the fixture"
    assert (mdg.digest(inp) if inp is not None else "") == str(d["input_photon_sha256"])
    assert np.array_equal(gs.view(np.uint32), d["gs"].view(np.uint32))
    eng = E.Engine(arrays, record_photon=1, record_seq=1)
    eng.simulate(int(d["event_index"]), gs, inp)
    r = strict_compare(eng.photons(), eng.seq()["seqhis"], d["photon"], d["seqhis"])
    eng.close()
    assert r["photons"] >= 100_000
    _assert_production(name, r, d)


@pytest.fixture(scope="module")
def nofma_digests(E, tmp_path_factory):
    """Digests of every fixture's photons from the engine built with --fmad=false, in each kernel form (a child
    process loads that build)."""
    import os
    import subprocess
    import sys
    from importlib import import_module
    lib = import_module("eic_opticks_gb300.build").build(variant="nofma")
    out = str(tmp_path_factory.mktemp("nofma") / "digests.npz")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, GBO_ENGINE_LIBRARY=lib)
    subprocess.run([sys.executable, os.path.join(root, "tests", "nofma_run.py"), out], env=env, check=True,
                   timeout=1800)
    return np.load(out)


@pytest.mark.parametrize("name", SIM_FIXTURES + CONFIGS)
def test_arithmetic_bit_exact_with_reference_device(nofma_digests, name):
    """The strict gate: without multiply-add contraction on either side, the engine's photons (record and flag
    history) equal the reference's bit for bit, in every kernel form (pool over pregenerated photons, one thread
    per photon, pool generating its photons, wavefront; Philox inlined or by call)."""
    want = _device_golden(name, "nofma")["digest"]
    for form in ("mode2", "mode1", "mode0", "mode3", "mode2_call", "mode1_call", "mode3_call"):
        got = nofma_digests["%s_%s" % (name, form)]
        assert len(got) == len(want)
        exact = float((got == want).mean()) if len(want) else 1.0
        print("%s kernel %s: %d photons, bit-exact %.6f" % (name, form, len(want), exact))
        assert exact >= 0.999


@pytest.mark.parametrize("keep_photon", [1, 0])
def test_hits_in_photon_order(E, keep_photon):
    z = load_golden("sim_crystal_array.npz")
    arrays = golden_arrays(z)
    eng = E.Engine(arrays, record_photon=keep_photon, record_seq=0)
    n = eng.simulate(int(z["event_index"]), z["gs"])
    hits = eng.hits()
    ref = z["photon"]
    want = ref[(ref["flagmask"] & (1 << 6)) != 0]
    assert n == len(hits)
    # order: photon index strictly increasing, identical to copy_if order
    assert np.all(np.diff(hits["index"].astype(np.int64)) > 0)
    common = np.intersect1d(hits["index"], want["index"])
    assert len(common) >= 0.99 * len(want)
    eng.close()


def test_facade_sequence(E):
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    ph = GS.isotropic_photons(1000, seed=5)
    gx = E.G4CXOpticks.SetGeometry(G.nested_boxes(sensor=True).arrays())
    E.SEvt.SetInputPhoton(ph)
    gx.simulate(0, reset=False)
    n = E.SEvt.GetNumHit(0)
    hits = E.SEvt.GetHits()
    assert n == len(hits) and n > 900
    assert np.all(hits["flagmask"] & (1 << 6))
    gx.reset(0)
    gx.engine.close()


def test_errors_are_reported(E):
    from eic_opticks_gb300 import geometry as G
    arrays = G.nested_boxes().arrays()
    eng = E.Engine(arrays)
    with pytest.raises(E.GBOError):
        eng.hits()                         # before any event
    gs = np.zeros((1, 6, 4), np.float32)
    gs.view(np.int32)[0, 0, 0] = 19        # INPUT_PHOTON genstep without photons
    gs.view(np.uint32)[0, 0, 3] = 10
    with pytest.raises(E.GBOError):
        eng.simulate(0, gs, None)
    eng.close()


def test_kernel_forms_agree(E):
    """The photon-pool kernel and the one-thread-per-photon kernel give every photon the same history, flags,
    indices and hits; float words agree within the reference-parity bounds (ptxas fuses mul+add into FMA per
    kernel, depending on each kernel's register budget, so their last bits can differ)."""
    z = load_golden("sim_crystal_array.npz")
    arrays = golden_arrays(z)
    outs = []
    forms = ((1, 1), (0, 1), (0, 8), (0, 32), (2, 1), (2, 8))
    for mode, refill in forms:
        eng = E.Engine(arrays, record_photon=1, record_seq=1, kernel_mode=mode, refill_min=refill)
        n = eng.simulate(int(z["event_index"]), z["gs"])
        outs.append((eng.photons(), eng.seq(), eng.hits(), n))
        eng.close()
    p0, s0, h0, n0 = outs[0]
    for p, s, h, n in outs[1:]:
        assert np.array_equal(s.view(np.uint64), s0.view(np.uint64))
        print("kernel forms: max |dpos| %.3g mm, |dt| %.3g ns, |dvec| %.3g, |dwl| %.3g" % assert_photons_agree(p, p0))
        assert n == n0 and np.array_equal(h["index"], h0["index"])
    # one compiled kernel gives the same bytes whatever its refill setting (which lane runs a photon, and when,
    # does not change the photon)
    for a, b in (((0, 1), (0, 32)), ((2, 1), (2, 8))):
        pa, pb = outs[forms.index(a)], outs[forms.index(b)]
        assert np.array_equal(pa[0].view(np.uint32), pb[0].view(np.uint32))
        assert np.array_equal(pa[2].view(np.uint32), pb[2].view(np.uint32))


@pytest.mark.parametrize("max_slot", [500, 1000, 1234])
def test_sliced_event_equals_whole(E, max_slot):
    """An event cut into launches of at most max_slot photons (OPTICKS_MAX_SLOT) gives the whole event's bytes."""
    z = load_golden("sim_crystal_array.npz")
    arrays = golden_arrays(z)
    whole = E.Engine(arrays, record_photon=1, record_seq=1)
    n0 = whole.simulate(2, z["gs"])
    p0, s0, h0 = whole.photons(), whole.seq(), whole.hits()
    whole.close()
    sliced = E.Engine(arrays, record_photon=1, record_seq=1, max_slot=max_slot)
    n1 = sliced.simulate(2, z["gs"])
    assert sliced.stats()["simulate_launches"] > 1
    assert n1 == n0
    assert np.array_equal(sliced.photons().view(np.uint32), p0.view(np.uint32))
    assert np.array_equal(sliced.seq().view(np.uint64), s0.view(np.uint64))
    assert np.array_equal(sliced.hits().view(np.uint32), h0.view(np.uint32))
    sliced.close()


@pytest.mark.parametrize("kernel_mode", [2, 3])
def test_simulate_to_host_equals_simulate_and_copy(E, kernel_mode):
    """gbo_simulate_to_host: the hits of gbo_simulate + gbo_copy_hits, for events of one launch and a max_slot-sliced
    event (each slice's hits copied out as it ends); a buffer smaller than the hit count keeps the first hits and the
    call reports the full count."""
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    arrays = G.crystal_array().arrays()
    small = GS.crystal_scint_gensteps(60, 900, seed=21)
    big = GS.crystal_scint_gensteps(400, 5000, seed=22)
    for gs, cfg in ((small, {}), (big, {}), (small, {"max_slot": 9000})):
        eng = E.Engine(arrays, kernel_mode=kernel_mode, **cfg)
        n0 = eng.simulate(5, gs)
        h0 = eng.hits()
        out = np.zeros(n0 + 3, dtype=E.L.PHOTON)
        n1 = eng.simulate_to_host(5, gs, out)
        st = eng.stats()
        assert n1 == n0 and np.array_equal(out[:n1].view(np.uint32), h0.view(np.uint32))
        assert np.array_equal(eng.hits().view(np.uint32), h0.view(np.uint32))
        if cfg:
            assert st["simulate_launches"] > 1
        short = np.zeros(n0 // 2, dtype=E.L.PHOTON)
        with pytest.raises(E.GBOError, match=r"code 4"):
            eng.simulate_to_host(5, gs, short)
        assert eng.num_hit() == n0
        assert np.array_equal(short.view(np.uint32), h0[:len(short)].view(np.uint32))
        eng.close()


def test_shards_on_separate_launches_equal_whole(E):
    """Event shards simulated as separate launches (as on separate GPUs) concatenate to the whole event's hits."""
    from eic_opticks_gb300 import geometry as G, gensteps as GS, shard
    arrays = G.crystal_array().arrays()
    gs = GS.crystal_scint_gensteps(50, 800, seed=12)
    eng = E.Engine(arrays)
    eng.simulate(7, gs)
    whole = eng.hits()
    parts = []
    for rank in range(3):
        part, offset = shard.shard_gensteps(gs, rank, 3)
        eng.simulate_slice(7, part, offset)
        parts.append(eng.hits())
    eng.close()
    merged = shard.merge_hits(parts)
    assert np.array_equal(merged.view(np.uint32), whole.view(np.uint32))
