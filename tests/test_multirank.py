"""Multi-rank event sharding, on CPU: two gloo ranks each simulate a contiguous genstep share of one event with
the oracle (photons indexed from the share's event offset), gather hits to rank 0, and reproduce the single-rank
event exactly.  This covers the host logic of splitting an event across GPUs without a GPU."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def rank_main(rank, world, port, result_path):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import __graft_entry__ as ge
    ge.load_package()
    O = ge.load_oracle()
    from eic_opticks_gb300 import geometry as G, gensteps as GS, shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    geom = G.crystal_array().arrays()
    gs = GS.crystal_scint_gensteps(9, 60, seed=31)
    part, offset = shard.shard_gensteps(gs, rank, world)
    cfg = O.SimConfig(geom)
    photons, _ = O.simulate(cfg, part, photon_offset=offset, event_index=4, seq=False)
    hits = photons[(photons["flagmask"] & (1 << 6)) != 0]
    gathered = [None] * world
    dist.all_gather_object(gathered, (offset, photons, hits))
    if rank == 0:
        all_photons = np.concatenate([g[1] for g in gathered])
        all_hits = shard.merge_hits([g[2] for g in gathered])
        np.savez(result_path, photons=all_photons, hits=all_hits, offsets=np.array([g[0] for g in gathered]))
    dist.barrier()
    dist.destroy_process_group()


def test_shard_ranges_cover_event():
    import __graft_entry__ as ge
    ge.load_package()
    from eic_opticks_gb300 import gensteps as GS, shard
    gs = GS.crystal_scint_gensteps(37, 300, seed=2)
    counts = shard.photon_counts(gs)
    for world in (1, 2, 3, 8):
        rs = shard.shard_ranges(gs, world)
        assert rs[0][0] == 0 and rs[-1][1] == len(gs)
        for (a0, a1, off), (b0, b1, _) in zip(rs, rs[1:]):
            assert a1 == b0
        for g0, g1, off in rs:
            assert off == counts[:g0].sum()


def test_two_gloo_ranks_reproduce_single_rank(tmp_path, oracle):
    import torch.multiprocessing as mp
    result = str(tmp_path / "r.npz")
    port = free_port()
    ctx = mp.get_context("spawn")
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, result)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    z = np.load(result)
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    gs = GS.crystal_scint_gensteps(9, 60, seed=31)
    whole, _ = oracle.simulate(oracle.SimConfig(G.crystal_array().arrays()), gs, event_index=4, seq=False)
    assert z["offsets"][1] > 0
    assert np.array_equal(z["photons"].view(np.uint32), whole.view(np.uint32))
    want_hits = whole[(whole["flagmask"] & (1 << 6)) != 0]
    assert np.array_equal(z["hits"].view(np.uint32), want_hits.view(np.uint32))
