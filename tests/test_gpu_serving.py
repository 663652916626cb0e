"""Continuous batching: every served event's hits equal those of the same event simulated alone, whatever it was
batched with, with events submitted concurrently from several threads."""
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import __graft_entry__ as ge
    ge.build()
    from eic_opticks_gb300 import engine
    return engine


def make_events(rng, n, geom_kind, wc=None):
    from eic_opticks_gb300 import gensteps as GS
    events = []
    for k in range(n):
        photons = int(10 ** rng.uniform(3, 5.3))               # log-uniform 1e3 .. 2e5 photons
        if geom_kind == "crystal":
            n_gs = max(1, photons // 500)
            gs = GS.crystal_scint_gensteps(n_gs, 500, seed=1000 + k, poisson=True)
        else:
            gs = GS.water_cerenkov_gensteps(wc, max(1, photons // 100), seed=2000 + k)
        events.append((100 + k, gs))
    return events


@pytest.mark.parametrize("kind,use_graph,mode", [("crystal", 1, 0), ("water", 1, 0), ("crystal", 0, 0), ("crystal", 1, 2),
                                                 ("crystal", 1, 3), ("water", 0, 3)])
def test_served_events_equal_alone(E, kind, use_graph, mode):
    from eic_opticks_gb300 import geometry as G
    geom = G.crystal_array() if kind == "crystal" else G.water_cube()
    arrays = geom.arrays()
    events = make_events(np.random.default_rng(7), 40, kind, wc=geom if kind == "water" else None)
    eng_alone = E.Engine(arrays, kernel_mode=mode)       # the same compiled kernel form as the server's
    alone = {}
    for eid, gs in events:
        eng_alone.simulate(eid, gs)
        alone[eid] = eng_alone.hits()
    eng_alone.close()

    eng = E.Engine(arrays, kernel_mode=mode)
    srv = E.Server(eng, slots=3, max_batch_events=16, use_graph=use_graph)
    tickets = {}
    lock = threading.Lock()

    def producer(chunk):
        for eid, gs in chunk:
            t = srv.submit(eid, gs)
            with lock:
                tickets[eid] = t

    threads = [threading.Thread(target=producer, args=(events[i::4],)) for i in range(4)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for eid, t in tickets.items():
        assert srv.wait(t, timeout_us=60_000_000)
        got = srv.hits(t)
        want = alone[eid]
        assert len(got) == len(want), eid
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), eid
        info = srv.info(t)
        assert info["latency_s"] > 0 and info["num_hit"] == len(want)
        srv.release(t)
    st = srv.stats()
    assert st["events_done"] == len(events) and st["batches"] < len(events)   # events were really packed
    assert st["graph_launches"] == (st["batches"] if use_graph else 0)
    if use_graph:       # one instantiation per slot; later batches update it in place
        print("batches %d, graph instantiations %d" % (st["batches"], st["graph_instantiations"]))
        assert 1 <= st["graph_instantiations"] <= 3
    srv.close()
    eng.close()


@pytest.mark.parametrize("max_batch_photon", [1200, 400])
def test_server_slices_events_larger_than_a_batch(E, max_batch_photon):
    """Events above max_batch_photon run as genstep-aligned pieces (several batches, both slots); each event's hits
    equal those it gets alone.  At 400 every 500-photon genstep is a piece of its own."""
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    arrays = G.crystal_array().arrays()
    events = [(300 + k, GS.crystal_scint_gensteps(10, 500, seed=70 + k, poisson=False)) for k in range(6)]
    eng = E.Engine(arrays)
    alone = {}
    for eid, gs in events:
        eng.simulate(eid, gs)
        alone[eid] = eng.hits()
    srv = E.Server(eng, slots=2, max_batch_photon=max_batch_photon)
    tickets = {eid: srv.submit(eid, gs) for eid, gs in events}
    for eid, t in tickets.items():
        assert srv.wait(t, timeout_us=60_000_000)
        got = srv.hits(t)
        assert np.array_equal(got.view(np.uint32), alone[eid].view(np.uint32)), eid
        assert srv.info(t)["num_photon"] == 5000
        srv.release(t)
    st = srv.stats()
    assert st["events_done"] == len(events) and st["photons"] == 5000 * len(events)
    assert st["batches"] >= len(events) * 5000 // 1200
    srv.close()
    eng.close()


@pytest.mark.parametrize("max_batch_photon", [16 << 20, 3000])
def test_server_input_photons(E, max_batch_photon):
    """INPUT_PHOTON events (nested boxes with the sensor surface): batched, and sliced into pieces, each event's
    hits equal those it gets alone."""
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    arrays = G.nested_boxes(sensor=True).arrays()
    events = []
    for k in range(8):
        inp = GS.isotropic_photons(2000 + 500 * k, seed=40 + k)
        q = len(inp) // 4                       # four INPUT_PHOTON gensteps, so that slicing can cut the event
        gs = np.concatenate([GS.input_photon_genstep(q)] * 3 + [GS.input_photon_genstep(len(inp) - 3 * q)])
        events.append((400 + k, gs, inp))
    eng = E.Engine(arrays)
    alone = {}
    for eid, gs, inp in events:
        eng.simulate(eid, gs, inp)
        alone[eid] = eng.hits()
    assert sum(len(h) for h in alone.values()) > 0
    srv = E.Server(eng, slots=2, max_batch_photon=max_batch_photon)
    tickets = {eid: srv.submit(eid, gs, inp) for eid, gs, inp in events}
    for eid, t in tickets.items():
        assert srv.wait(t, timeout_us=60_000_000)
        assert np.array_equal(srv.hits(t).view(np.uint32), alone[eid].view(np.uint32)), eid
        srv.release(t)
    srv.close()
    eng.close()


def test_event_api_on_engine_handle(E):
    """gbo_event_submit / wait / num_hits / copy_hits / release on the engine handle, from three producer threads:
    each event's hits equal those of gbo_simulate with the same event id."""
    import ctypes as C
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    arrays = G.crystal_array().arrays()
    events = [(500 + k, GS.crystal_scint_gensteps(4 + k, 700, seed=90 + k)) for k in range(9)]
    alone_eng = E.Engine(arrays)
    alone = {}
    for eid, gs in events:
        alone_eng.simulate(eid, gs)
        alone[eid] = alone_eng.hits()
    alone_eng.close()
    eng = E.Engine(arrays)
    lib = eng.lib
    lib.gbo_event_num_hits.restype = C.c_int64
    tickets, lock = {}, threading.Lock()

    def producer(chunk):
        for eid, gs in chunk:
            t = C.c_uint64()
            g = np.ascontiguousarray(gs)
            rc = lib.gbo_event_submit(eng.handle, g.ctypes.data_as(C.c_void_p), C.c_size_t(len(g)), C.c_uint32(eid),
                                      C.byref(t))
            assert rc == 0
            with lock:
                tickets[eid] = t.value

    threads = [threading.Thread(target=producer, args=(events[i::3],)) for i in range(3)]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for eid, t in tickets.items():
        assert lib.gbo_event_wait(eng.handle, C.c_uint64(t), C.c_int64(60_000_000_000)) == 0
        n = lib.gbo_event_num_hits(eng.handle, C.c_uint64(t))
        assert n == len(alone[eid])
        got = np.zeros(n, dtype=alone[eid].dtype)
        assert lib.gbo_event_copy_hits(eng.handle, C.c_uint64(t), got.ctypes.data_as(C.c_void_p), C.c_size_t(n)) == 0
        assert np.array_equal(got.view(np.uint32), alone[eid].view(np.uint32)), eid
        assert lib.gbo_event_release(eng.handle, C.c_uint64(t)) == 0
    eng.close()
