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


@pytest.mark.parametrize("kind,use_graph", [("crystal", 1), ("water", 1), ("crystal", 0)])
def test_served_events_equal_alone(E, kind, use_graph):
    from eic_opticks_gb300 import geometry as G
    geom = G.crystal_array() if kind == "crystal" else G.water_cube()
    arrays = geom.arrays()
    events = make_events(np.random.default_rng(7), 40, kind, wc=geom if kind == "water" else None)
    eng_alone = E.Engine(arrays)
    alone = {}
    for eid, gs in events:
        eng_alone.simulate(eid, gs)
        alone[eid] = eng_alone.hits()
    eng_alone.close()

    eng = E.Engine(arrays)
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


def test_server_rejects_oversized_event(E):
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    eng = E.Engine(G.crystal_array().arrays())
    srv = E.Server(eng, max_batch_photon=1000)
    with pytest.raises(E.GBOError):
        srv.submit(0, GS.crystal_scint_gensteps(4, 500, seed=1, poisson=False))
    srv.close()
    eng.close()
