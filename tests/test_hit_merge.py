"""Hit merging by (sensor identity, time bucket): the reference's SPM::merge_partial_select semantics
(sysrap/SPM.cu, sysrap/sphoton.h:277-304).  Pinned by tests/golden/merge.npz, written by the reference's own
select / key / reduce functors run through thrust (oracle/ref_spm.cc, tests/golden/make_merge_golden.py): the
oracle (orc_qsim.c) and the GPU merge (gbo_merge.cu) reproduce it byte for byte; a second, numpy restatement and
synthetic cases at scale cross-check the oracle and the GPU merge against each other."""
import numpy as np
import pytest

from conftest import golden_arrays, load_golden


def synthetic_hits(n, num_ids, t_max, seed):
    from eic_opticks_gb300 import layout as L
    rng = np.random.default_rng(seed)
    h = np.zeros(n, dtype=L.PHOTON)
    h["pos"] = rng.normal(size=(n, 3)).astype(np.float32)
    h["time"] = rng.uniform(0, t_max, n).astype(np.float32)
    h["time"][rng.integers(0, n, n // 50)] = 3.0                 # exact ties inside one bucket
    h["identity"] = rng.integers(1, num_ids + 1, n).astype(np.uint32) | (rng.integers(0, 2, n).astype(np.uint32) << 24)
    h["hitcount_iindex"] = (1 << 16) | rng.integers(0, 65536, n).astype(np.uint32)
    h["flagmask"] = (1 << 6) | rng.integers(0, 1 << 12, n).astype(np.uint32)
    h["index"] = np.arange(n, dtype=np.uint32)
    return h


def numpy_merge(h, tw):
    """Second restatement: stable argsort of the keys, then a fold per run."""
    key = (h["identity"].astype(np.uint64) & np.uint64(0xFFFFFF)) << np.uint64(48)
    key |= (h["time"] / np.float32(tw)).astype(np.uint32).astype(np.uint64)
    order = np.argsort(key, kind="stable")
    out = []
    k = key[order]
    starts = np.flatnonzero(np.r_[True, k[1:] != k[:-1]])
    ends = np.r_[starts[1:], len(k)]
    for b, e in zip(starts, ends):
        idx = order[b:e]
        t = h["time"][idx]
        first = idx[np.flatnonzero(t == t.min())[0]]
        r = h[first].copy()
        r["flagmask"] = np.bitwise_or.reduce(h["flagmask"][idx])
        hc = int((h["hitcount_iindex"][idx] >> 16).astype(np.int64).sum()) & 0xFFFF
        r["hitcount_iindex"] = (int(r["hitcount_iindex"]) & 0xFFFF) | (hc << 16)
        out.append(r)
    return np.array(out, dtype=h.dtype)


MERGE_CASES = [("crystal", 0.0), ("crystal", 1.0), ("crystal", 10.0), ("large_sphere", 0.0), ("large_sphere", 1.0),
               ("large_sphere", 10.0), ("synthetic", 0.0), ("synthetic", 1.0), ("synthetic", 10.0),
               ("synthetic", 0.37)]


@pytest.mark.parametrize("case,tw", MERGE_CASES)
def test_oracle_merge_matches_reference_functors(oracle, case, tw):
    z = load_golden("merge.npz")
    hits, want = z[case + "_hits"], z["%s_tw%g" % (case, tw)]
    got = oracle.merge_hits(hits, tw)
    assert len(got) == len(want) and np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.parametrize("tw", [1.0, 0.37, 25.0])
def test_oracle_merge_matches_numpy(oracle, tw):
    h = synthetic_hits(20000, 300, 200.0, seed=4)
    a = oracle.merge_hits(h, tw)
    b = numpy_merge(h, tw)
    assert len(a) == len(b) and np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert (a["hitcount_iindex"] >> 16).sum() == len(h)          # every hit counted once (no 16-bit wrap here)


def test_oracle_merge_window_zero_keeps_hits(oracle):
    h = synthetic_hits(500, 10, 50.0, seed=1)
    assert np.array_equal(oracle.merge_hits(h, 0.0).view(np.uint32), h.view(np.uint32))


@pytest.fixture(scope="module")
def E():
    import __graft_entry__ as ge
    ge.build()
    from eic_opticks_gb300 import engine
    return engine


@pytest.mark.gpu
@pytest.mark.parametrize("case,tw", MERGE_CASES)
def test_device_merge_matches_reference_functors(E, case, tw):
    """gbo_merge_hits_device against the reference functors' output, byte for byte."""
    import ctypes as C
    import torch
    z = load_golden("merge.npz")
    h, want = z[case + "_hits"], z["%s_tw%g" % (case, tw)]
    lib = E.load()
    d_in = torch.from_numpy(h.view(np.uint8).copy()).cuda()
    d_out = torch.zeros_like(d_in)
    m = C.c_int64()
    rc = lib.gbo_merge_hits_device(C.c_void_p(d_in.data_ptr()), len(h), C.c_float(tw), C.c_void_p(d_out.data_ptr()),
                                   C.byref(m), None)
    assert rc == 0
    got = d_out.cpu().numpy()[: m.value * h.dtype.itemsize].view(h.dtype)
    print("%s window %g: %d hits -> %d" % (case, tw, len(h), len(got)))
    assert len(got) == len(want) and np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.gpu
@pytest.mark.parametrize("tw", [1.0, 10.0, 0.0])
def test_engine_merge_matches_oracle(E, oracle, tw):
    z = load_golden("sim_large_sphere_small.npz")
    eng = E.Engine(golden_arrays(z))
    eng.simulate(int(z["event_index"]), z["gs"])
    hits = eng.hits()
    got = eng.merge_hits(tw)
    want = oracle.merge_hits(hits, tw)
    print("tw %g: %d hits -> %d merged" % (tw, len(hits), len(got)))
    assert len(hits) > 0 and np.array_equal(got.view(np.uint32), want.view(np.uint32))
    eng.close()


@pytest.mark.gpu
@pytest.mark.parametrize("n,num_ids,t_max", [(1, 1, 1.0), (4097, 3, 5.0), (300000, 20000, 400.0), (2_000_000, 70000, 3000.0)])
def test_device_merge_matches_oracle(E, oracle, n, num_ids, t_max):
    """Synthetic hits through gbo_merge_hits_device: ragged tile edges, identities above 16 bits (the reference's
    64-bit key drops the top 8), wide time ranges (more radix passes), ties."""
    import ctypes as C
    import torch
    h = synthetic_hits(n, num_ids, t_max, seed=n)
    lib = E.load()
    d_in = torch.from_numpy(h.view(np.uint8).copy()).cuda()
    d_out = torch.zeros_like(d_in)
    m = C.c_int64()
    rc = lib.gbo_merge_hits_device(C.c_void_p(d_in.data_ptr()), n, C.c_float(1.0), C.c_void_p(d_out.data_ptr()),
                                   C.byref(m), None)
    assert rc == 0
    got = d_out.cpu().numpy()[: m.value * h.dtype.itemsize].view(h.dtype)
    want = oracle.merge_hits(h, 1.0)
    assert len(got) == len(want) and np.array_equal(got.view(np.uint32), want.view(np.uint32))


@pytest.mark.gpu
def test_device_merge_unaligned_buffers(E, oracle):
    """Hit arrays that start 4 bytes past a 16-byte boundary take the 4-byte load path of the run fold."""
    import ctypes as C
    import torch
    n = 50000
    h = synthetic_hits(n, 900, 60.0, seed=5)
    lib = E.load()
    raw_in = torch.zeros(h.nbytes + 16, dtype=torch.uint8, device="cuda")
    raw_in[4: 4 + h.nbytes] = torch.from_numpy(h.view(np.uint8).copy()).cuda()
    raw_out = torch.zeros_like(raw_in)
    m = C.c_int64()
    rc = lib.gbo_merge_hits_device(C.c_void_p(raw_in.data_ptr() + 4), n, C.c_float(1.0),
                                   C.c_void_p(raw_out.data_ptr() + 4), C.byref(m), None)
    assert rc == 0
    got = raw_out.cpu().numpy()[4: 4 + m.value * h.dtype.itemsize].view(h.dtype)
    want = oracle.merge_hits(h, 1.0)
    assert len(got) == len(want) and np.array_equal(got.view(np.uint32), want.view(np.uint32))
