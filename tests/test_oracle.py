"""Pin the CPU oracle against the reference.

Two sources pin it:
* golden fixtures in tests/golden/, written by tests/golden/make_golden.py from the reference's own headers
  compiled for the host (oracle/_ref) and curand's host Philox;
* the reference build itself, when oracle/_ref/libref.so is present (this container), on fresh random inputs.

The bar is bit-exact: the oracle is a binary32 restatement in the reference's operation order.
"""
import numpy as np
import pytest

from conftest import CSG_SHAPES, SIM_FIXTURES, golden_arrays, load_golden


def test_philox_matches_curand_golden(oracle):
    z = load_golden("philox.npz")
    for case, want in zip(z["cases"], z["uniforms"]):
        got = oracle.philox_uniforms(int(case[0]), int(case[1]), int(case[2]), int(case[3]), want.shape[0])
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), case


def test_philox_uniform_range(oracle):
    u = oracle.philox_uniforms(0, 12345, 0, 0, 100000)
    assert u.min() > 0.0 and u.max() <= 1.0
    assert abs(u.mean() - 0.5) < 0.005


@pytest.mark.parametrize("name", CSG_SHAPES)
def test_csg_intersect_golden(oracle, name):
    z = load_golden("csg.npz")
    node, itra, plan = z[name + "_node"], z[name + "_itra"], z[name + "_plan"]
    o, d, want, valid = z[name + "_o"], z[name + "_d"], z[name + "_isect"], z[name + "_valid"]
    for i in range(len(o)):
        v, got = oracle.intersect_prim(node, plan, itra, 0.05, o[i], d[i])
        assert v == bool(valid[i]), (name, i)
        assert np.array_equal(got.view(np.uint32), want[i].view(np.uint32)), (name, i, got, want[i])


@pytest.mark.parametrize("name", SIM_FIXTURES)
def test_simulate_golden(oracle, name):
    z = load_golden("sim_%s.npz" % name)
    cfg = oracle.SimConfig(golden_arrays(z))
    inp = z["input_photon"] if len(z["input_photon"]) else None
    out, seq = oracle.simulate(cfg, z["gs"], inp, event_index=int(z["event_index"]), nthreads=4)
    want = z["photon"]
    assert out.shape == want.shape
    same = np.all(out.view(np.uint32).reshape(-1, 16) == want.view(np.uint32).reshape(-1, 16), axis=1)
    assert same.all(), np.where(~same)[0][:10]
    assert np.array_equal(seq.view(np.uint64), z["seq"].view(np.uint64))


def test_simulate_threads_invariant(oracle):
    z = load_golden("sim_crystal_array.npz")
    cfg = oracle.SimConfig(golden_arrays(z))
    a, sa = oracle.simulate(cfg, z["gs"], nthreads=1)
    b, sb = oracle.simulate(cfg, z["gs"], nthreads=7)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_hit_selection_order(oracle):
    """Hits are the photons with every hitmask bit set, in photon order (sysrap/sphoton.h:1219-1225)."""
    import ctypes as C
    z = load_golden("sim_nested_boxes_sensor.npz")
    p = np.ascontiguousarray(z["photon"])
    hits = np.zeros_like(p)
    n = oracle.lib().orc_select_hits(p.ctypes.data_as(C.c_void_p), C.c_int64(len(p)), C.c_uint32(1 << 6),
                                     hits.ctypes.data_as(C.c_void_p))
    sel = p[(p["flagmask"] & (1 << 6)) == (1 << 6)]
    assert n == len(sel) > 0
    assert np.array_equal(hits[:n].view(np.uint32), sel.view(np.uint32))


@pytest.fixture(scope="module")
def ref(oracle):
    import os
    ref = os.environ.get("GBO_REFERENCE_DIR")
    if not ref or not os.path.isdir(os.path.join(ref, "qudarap")):
        pytest.skip("reference tree not available (GBO_REFERENCE_DIR)")
    oracle.build(ref=True)
    if oracle.reflib() is None:
        pytest.skip("reference build not available")
    return oracle


def test_philox_matches_curand_live(ref):
    rng = np.random.default_rng(0)
    for _ in range(50):
        seed, sub = int(rng.integers(0, 2**63)), int(rng.integers(0, 2**63))
        off, skip = int(rng.integers(0, 1000)), int(rng.integers(0, 10**9))
        a = ref.philox_uniforms(seed, sub, off, skip, 13)
        b = ref.philox_uniforms(seed, sub, off, skip, 13, use_ref=True)
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_simulate_matches_reference_live(ref):
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    g = G.crystal_array()
    cfg = ref.SimConfig(g.arrays())
    gs = GS.crystal_scint_gensteps(6, 80, seed=123)
    a, sa = ref.simulate(cfg, gs, event_index=2)
    b, sb = ref.simulate(cfg, gs, event_index=2, use_ref=True)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert np.array_equal(sa.view(np.uint64), sb.view(np.uint64))
