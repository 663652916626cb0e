"""gbo_autotune: the project's tuner of the kernel form (kernel mode, refill threshold, compaction period, resident
blocks per SM, lanes gathered per TLAS walk, Philox blocks by call).  It keeps the fastest candidate it measured, and no candidate changes any photon's history, flags,
index or hit decision (a kernel form decides only which lane runs a photon, and when)."""
import numpy as np
import pytest

from conftest import assert_forms_agree, golden_arrays, load_golden


pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def E():
    import __graft_entry__ as ge
    ge.build()
    from eic_opticks_gb300 import engine
    return engine


@pytest.mark.parametrize("fixture", ["sim_crystal_array.npz", "sim_large_sphere_small.npz"])
def test_autotune_keeps_fastest_and_results_unchanged(E, fixture):
    z = load_golden(fixture)
    arrays = golden_arrays(z)
    eng = E.Engine(arrays)
    r = eng.autotune(0, z["gs"], trials=2)
    cands = r["candidates"]
    ms = np.array([c["ms"] for c in cands])
    best = cands[int(np.argmin(ms))]
    print("%s: %d candidates, fastest %.3f ms (mode %d refill %d period %d blocks %d walk %d rng_call %d), slowest "
          "%.3f ms" % (fixture, len(cands), ms.min(), best["mode"], best["refill"], best["period"],
                       best["blocks_per_sm"], best["walk_min"], best["rng_call"], ms.max()))
    key = ("mode", "refill", "period", "blocks_per_sm", "walk_min", "rng_call")
    assert (r["kernel_mode"], r["refill_min"], r["refill_period"], r["blocks_per_sm"], r["walk_min"],
            r["rng_call"]) == tuple(best[k] for k in key)
    assert any(c["blocks_per_sm"] > 0 for c in cands)          # block shapes are among the candidates
    assert any(c["mode"] == 3 for c in cands)                  # and the wavefront form
    if fixture == "sim_crystal_array.npz":                     # and, without CSG trees, Philox by call
        assert any(c["rng_call"] for c in cands)
    else:                                                      # with CSG trees, gathered TLAS walks
        assert any(c["walk_min"] > 1 for c in cands)
    assert len({tuple(c[k] for k in key) for c in cands}) == len(cands)
    eng.close()
    # every candidate form gives the same photons (histories, flags, indices, hits exactly; floats within a few ulp
    # between separately compiled kernels)
    ref = None
    for c in cands:
        eng = E.Engine(arrays, record_photon=1, record_seq=1, kernel_mode=c["mode"], refill_min=c["refill"],
                       refill_period=c["period"], blocks_per_sm=c["blocks_per_sm"], walk_min=c["walk_min"],
                       rng_call=c["rng_call"])
        eng.simulate(int(z["event_index"]), z["gs"])
        got = (eng.photons(), eng.seq(), eng.hits())
        eng.close()
        if ref is None:
            ref = got
            continue
        assert np.array_equal(got[1].view(np.uint64), ref[1].view(np.uint64))
        assert np.array_equal(got[2]["index"], ref[2]["index"])
        assert_forms_agree(got[0], ref[0], fixture)
