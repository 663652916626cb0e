"""Edge cases the reference's event loop meets: empty events, gensteps with no photons, empty server events,
input-photon events cut into launches, events larger than the photon limit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import __graft_entry__ as ge
    ge.build()
    from eic_opticks_gb300 import engine
    return engine


def test_empty_event(E):
    from eic_opticks_gb300 import geometry as G
    eng = E.Engine(G.crystal_array().arrays())
    assert eng.simulate(0, np.zeros((0, 6, 4), np.float32)) == 0
    assert len(eng.hits()) == 0 and eng.num_photon() == 0
    assert len(eng.merge_hits(1.0)) == 0
    eng.close()


def test_zero_photon_gensteps_change_nothing(E):
    """Gensteps with numphoton 0 interleaved with real ones: the same photons (indices, random streams) and hits."""
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    arrays = G.crystal_array().arrays()
    gs = GS.crystal_scint_gensteps(12, 300, seed=8, poisson=False)
    empty = gs[:1].copy()
    empty.view(np.uint32)[0, 0, 3] = 0
    mixed = np.concatenate([empty, gs[:5], empty, empty, gs[5:], empty])
    eng = E.Engine(arrays)
    n0 = eng.simulate(4, gs)
    h0 = eng.hits()
    n1 = eng.simulate(4, mixed)
    h1 = eng.hits()
    eng.close()
    assert n0 == n1 > 0 and np.array_equal(h0.view(np.uint32), h1.view(np.uint32))


def test_server_empty_and_zero_photon_events(E):
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    eng = E.Engine(G.crystal_array().arrays())
    srv = E.Server(eng, slots=2)
    gs = GS.crystal_scint_gensteps(3, 200, seed=9, poisson=False)
    zero = gs.copy()
    zero.view(np.uint32)[:, 0, 3] = 0
    t_empty = srv.submit(1, np.zeros((0, 6, 4), np.float32))
    t_zero = srv.submit(2, zero)
    t_real = srv.submit(3, gs)
    for t in (t_empty, t_zero, t_real):
        assert srv.wait(t, timeout_us=30_000_000)
    assert srv.info(t_empty)["num_hit"] == 0 and srv.info(t_zero)["num_hit"] == 0
    eng.simulate(3, gs)
    assert np.array_equal(srv.hits(t_real).view(np.uint32), eng.hits().view(np.uint32))
    srv.close()
    eng.close()


@pytest.mark.parametrize("max_slot", [700, 2000])
def test_sliced_input_photon_event_equals_whole(E, max_slot):
    """OPTICKS_MAX_SLOT slicing of an INPUT_PHOTON event made of several gensteps: each slice reads its own input
    photons and keeps their event-level indices."""
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    arrays = G.nested_boxes(sensor=True).arrays()
    inp = GS.isotropic_photons(5000, seed=12)
    gs = np.concatenate([GS.input_photon_genstep(1000)] * 5)
    whole = E.Engine(arrays)
    whole.simulate(2, gs, inp)
    want = whole.hits()
    whole.close()
    sliced = E.Engine(arrays, max_slot=max_slot)
    sliced.simulate(2, gs, inp)
    got = sliced.hits()
    sliced.close()
    assert len(want) > 0 and np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_event_above_photon_limit_is_refused(E):
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    eng = E.Engine(G.crystal_array().arrays(), max_photon=1000)
    with pytest.raises(E.GBOError):
        eng.simulate(0, GS.crystal_scint_gensteps(4, 500, seed=1, poisson=False))
    assert eng.simulate(0, GS.crystal_scint_gensteps(1, 500, seed=1, poisson=False)) >= 0    # still usable
    eng.close()


@pytest.mark.parametrize("n_photon", [1, 31, 33, 1000, 4097])
def test_pregenerated_pool_small_events_equal_one_thread(E, n_photon):
    """The pregenerated photon pool hands photons out in warp chunks of 32, the wavefront appends them to its step
    lists a warp at a time: events smaller than one chunk, than the grid, and with ragged last chunks give the same
    photons and hits as the one-thread-per-photon kernel."""
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    arrays = G.crystal_array().arrays()
    gs = GS.crystal_scint_gensteps(1, n_photon, seed=n_photon, poisson=False)
    out = []
    for mode in (1, 2, 3):
        eng = E.Engine(arrays, record_photon=1, record_seq=1, kernel_mode=mode, refill_min=1)
        eng.simulate(5, gs)
        out.append((eng.photons(), eng.seq(), eng.hits()))
        eng.close()
    p1, s1, h1 = out[0]
    for p2, s2, h2 in out[1:]:
        assert len(p1) == len(p2) == n_photon
        assert np.array_equal(s1.view(np.uint64), s2.view(np.uint64))
        assert np.array_equal(p1["index"], p2["index"]) and np.array_equal(h1["index"], h2["index"])


@pytest.mark.parametrize("max_bounce", [0, 1, 2, 5])
def test_wavefront_bounce_limit(E, max_bounce):
    """The wavefront runs max_bounce steps; photons still alive after the last one end there, as the bounce loop of
    the other forms ends them: same flag histories, photons and hits for every limit, including none."""
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    arrays = G.crystal_array().arrays()
    gs = GS.crystal_scint_gensteps(4, 500, seed=3, poisson=False)
    out = []
    for mode in (1, 3):
        eng = E.Engine(arrays, record_photon=1, record_seq=1, kernel_mode=mode, max_bounce=max_bounce)
        eng.simulate(2, gs)
        out.append((eng.photons(), eng.seq(), eng.hits()))
        eng.close()
    (p1, s1, h1), (p3, s3, h3) = out
    assert np.array_equal(s1.view(np.uint64), s3.view(np.uint64))
    assert np.array_equal(p1["flagmask"], p3["flagmask"]) and np.array_equal(h1["index"], h3["index"])
    assert np.allclose(p1["pos"], p3["pos"], atol=1e-3)


def test_genstep_hint_outside_every_instance(E):
    """A genstep whose position lies outside every instance box gets no start hint; its photons still trace from
    the TLAS root and match the one-thread kernel."""
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    arrays = G.nested_boxes(sensor=True).arrays()
    gs = GS.input_photon_genstep(2000)
    gs.view(np.float32)[0, 1, :3] = 1e7          # q1.xyz: far outside the world box
    inp = GS.isotropic_photons(2000, seed=4)
    out = []
    for mode in (1, 2):
        eng = E.Engine(arrays, kernel_mode=mode)
        eng.simulate(0, gs, inp)
        out.append(eng.hits())
        eng.close()
    assert len(out[0]) > 0 and np.array_equal(out[0]["index"], out[1]["index"])
