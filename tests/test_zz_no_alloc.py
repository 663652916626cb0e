"""gbo_simulate_noalloc : the simulation entry point for callers that cannot allocate device memory per event.

Its hits must equal those of the allocating device entry point (gbo_simulate_device) for the same event: the same
photons, indices, flags and histories, float words within a few ulp (the no-allocation kernel is a separate kernel,
and ptxas fuses mul+add per kernel), and a repeated call must give the same bytes again, so that state left in the
shared scratch array by one call cannot leak into the next.  This file is collected last so that a run stopping at
the first failure has already run every other test; it also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import assert_photons_agree

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    import torch
    import __graft_entry__ as ge
    ge.build()
    from eic_opticks_gb300 import engine as E, geometry as G, gensteps as GS
    lib = E.load()
    lib.gbo_simulate_noalloc.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                         C.c_void_p, C.c_int64, C.POINTER(C.c_int64), C.c_void_p]
    lib.gbo_noalloc_scratch_bytes.restype = C.c_int64
    eng = E.Engine(G.crystal_array().arrays(), device=0)
    gs = GS.crystal_scint_gensteps(60, 1500, seed=21)
    d_gs = torch.from_numpy(gs.copy()).cuda()
    yield torch, E, lib, eng, gs, d_gs
    eng.close()


def noalloc_hits(torch, E, lib, eng, d_gs, n_gs, event_id, capacity):
    d_hits = torch.zeros((capacity, 16), dtype=torch.float32, device="cuda")
    n = C.c_int64(-1)
    rc = lib.gbo_simulate_noalloc(eng.handle, event_id, C.c_void_p(d_gs.data_ptr()), n_gs, None, 0,
                                  C.c_void_p(d_hits.data_ptr()), capacity, C.byref(n), None)
    return rc, n.value, d_hits


def test_scratch_is_modest(setup):
    torch, E, lib, eng, gs, d_gs = setup
    assert 0 < lib.gbo_noalloc_scratch_bytes() <= 16 << 20


def test_noalloc_matches_device_entry_point_twice(setup):
    torch, E, lib, eng, gs, d_gs = setup
    first = {}
    for event_id in (5, 6, 5):
        want_n = eng.simulate_device(event_id, d_gs.data_ptr(), len(gs))
        want = eng.hits()
        rc, n, d_hits = noalloc_hits(torch, E, lib, eng, d_gs, len(gs), event_id, 2 * want_n + 16)
        assert rc == 0, lib.gbo_last_error()
        assert n == want_n
        got = d_hits[:n].cpu().numpy().view(E.L.PHOTON).reshape(-1)
        print("no-alloc vs device entry point, event %d: max |dpos| %.3g mm, |dt| %.3g ns, |dvec| %.3g, |dwl| %.3g"
              % ((event_id,) + assert_photons_agree(got, want)))
        if event_id in first:
            assert np.array_equal(got.view(np.uint32), first[event_id])       # repeated call: same bytes
        first[event_id] = got.view(np.uint32).copy()


def test_noalloc_rejects_sizes_beyond_limits(setup):
    torch, E, lib, eng, gs, d_gs = setup
    too_many = 40000                      # above the 32768 genstep limit
    big = torch.zeros((too_many, 6, 4), dtype=torch.float32, device="cuda")
    rc, n, _ = noalloc_hits(torch, E, lib, eng, big, too_many, 0, 16)
    assert rc == 4 and b"genstep" in lib.gbo_last_error()
    rc, n, _ = noalloc_hits(torch, E, lib, eng, d_gs, len(gs), 5, 1)     # hit buffer too small
    assert rc == 4 and n > 1 and b"hit buffer" in lib.gbo_last_error()


def test_noalloc_rejects_photon_limit_before_simulating(setup):
    """One genstep of 5,000,000 photons is above the 4,194,304-photon limit: refused after the genstep prefix,
    before any photon is simulated (no hit is counted), and the next call is unaffected."""
    torch, E, lib, eng, gs, d_gs = setup
    big = gs[:1].copy()
    big.view(np.uint32)[0, 0, 3] = 5_000_000
    rc, n, _ = noalloc_hits(torch, E, lib, eng, torch.from_numpy(big).cuda(), 1, 0, 16)
    assert rc == 4 and b"photons above the limit" in lib.gbo_last_error() and n == 0
    want_n = eng.simulate_device(5, d_gs.data_ptr(), len(gs))
    rc, n, _ = noalloc_hits(torch, E, lib, eng, d_gs, len(gs), 5, 2 * want_n + 16)
    assert rc == 0 and n == want_n


def test_noalloc_refuses_input_photon_gensteps_without_photons(setup):
    """INPUT_PHOTON gensteps with no input-photon buffer are refused on the host (no device read through a null
    pointer), by this entry point and by the allocating device entry point alike."""
    torch, E, lib, eng, gs, d_gs = setup
    from eic_opticks_gb300 import gensteps as GS
    d_inp_gs = torch.from_numpy(GS.input_photon_genstep(100).copy()).cuda()
    rc, n, _ = noalloc_hits(torch, E, lib, eng, d_inp_gs, 1, 0, 16)
    assert rc == 1 and b"input photons" in lib.gbo_last_error()
    with pytest.raises(E.GBOError):
        eng.simulate_device(0, d_inp_gs.data_ptr(), 1)


def test_noalloc_staging_overflow_reports_count(setup):
    """More hits than the 131,072-hit staging area: GBO_ERR_CAPACITY with *num_hit holding the full count; the
    next, smaller call still matches the allocating entry point."""
    torch, E, lib, eng0, gs, d_gs = setup
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    eng = E.Engine(G.nested_boxes(sensor=True).arrays(), device=0)
    try:
        ph = GS.isotropic_photons(200_000, seed=8)
        d_ph = torch.from_numpy(ph.view(np.float32).reshape(-1, 16).copy()).cuda()
        d_pgs = torch.from_numpy(GS.input_photon_genstep(len(ph)).copy()).cuda()
        want_n = eng.simulate_device(2, d_pgs.data_ptr(), 1, d_ph.data_ptr(), len(ph))
        assert want_n > 131072
        d_hits = torch.zeros((16, 16), dtype=torch.float32, device="cuda")
        n = C.c_int64(-1)
        rc = lib.gbo_simulate_noalloc(eng.handle, 2, C.c_void_p(d_pgs.data_ptr()), 1, C.c_void_p(d_ph.data_ptr()),
                                      len(ph), C.c_void_p(d_hits.data_ptr()), 16, C.byref(n), None)
        assert rc == 4 and b"staging" in lib.gbo_last_error() and n.value == want_n
        small = GS.input_photon_genstep(5000)
        d_sgs = torch.from_numpy(small.copy()).cuda()
        want_n = eng.simulate_device(3, d_sgs.data_ptr(), 1, d_ph.data_ptr(), 5000)
        want = eng.hits()
        d_hits = torch.zeros((want_n + 16, 16), dtype=torch.float32, device="cuda")
        rc = lib.gbo_simulate_noalloc(eng.handle, 3, C.c_void_p(d_sgs.data_ptr()), 1, C.c_void_p(d_ph.data_ptr()),
                                      5000, C.c_void_p(d_hits.data_ptr()), want_n + 16, C.byref(n), None)
        assert rc == 0 and n.value == want_n
        got = d_hits[:want_n].cpu().numpy().view(E.L.PHOTON).reshape(-1)
        assert_photons_agree(got, want)
    finally:
        eng.close()
