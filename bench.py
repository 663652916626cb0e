"""Benchmark: propagated photons/s of the GB300 engine on the scintillating crystal-array workload.

Workload (one step = one event): the 8x8 CsI crystal array, 2,000 scintillation gensteps with Poisson(5000)
photons each (~10M photons), Gaussian 550+-50 nm emission through the 3x4096 hd_factor-20 inverse CDF,
1000 ns decay, reference physics defaults (max_bounce 31, epsilon 0.05 mm, hit mask SD), synthetic gensteps
from seeded numpy generators (Geant4 is not part of the path).

* ``value``  photons/s with the gensteps already resident in device memory (gbo_simulate_device), timed with
  CUDA events around each event; L2 is flushed (256 MB write) between timed events.
* ``e2e``    photons/s through the reference-facing C ABI (gbo_simulate_to_host: host gensteps in, the event's hits
  out into page-locked host memory), host<->device copies inside the timed region; ``e2e.two_calls`` is the same
  through gbo_simulate followed by gbo_copy_hits.
* ``roofline`` the simulate kernel's algorithmic HBM bytes per photon (genstep share + 4 B seed + 64 B photon
  write + 64 B compaction read + 64 B x hit fraction, the reference's traffic for the same event) over its
  CUDA-event time, against the measured copy bandwidth.
* ``cpu_baseline`` the CPU oracle (the reference's algorithm restated in C, pthreads over all host cores) on a
  bounded sample of the same event.

``--impl reference`` times the reference's CPU implementation of the path instead (oracle/_ref when it was
built from the reference's own headers on this host, else the oracle port), on the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

METRIC = "propagated photons/s, batched vs plain per-event launch on 1 GB300; p99 latency"
UNIT = "photons/s"
WORKLOAD = "crystal_array_8x8_CsI_scint_2000gs_poisson5000"
L2_FLUSH_BYTES = 256 << 20
# ncu DRAM bytes (read + write) per photon of the simulate kernels, scaled to the benchmark event by its photon count
# (all of it grows with the photons), each with the build it was captured on: one thread per photon on the crystal
# event (k_simulate, 1M photons: gensteps in, hits and hit bitmap out), the pregenerated pool on the crystal event
# (k_generate + k_simulate_pool, 2.5M photons: 0.33 + 197.31 MB and 211.36 + 2.20 MB, larger than L2) and the
# wavefront on the 20,000-sensor sphere (k_generate + k_wf_start + 31 x (3 passes + the walk-queue sort), 5M
# photons: 8942 MB)
TRAFFIC_B_PER_PHOTON = {("crystal_array", 1): (443392.0 + 840192.0) / 998319,
                        ("crystal_array", 2): (0.33e6 + 197.31e6 + 211.36e6 + 2.20e6) / 2499792,
                        ("large_sphere", 3): 8942.13e6 / 5000000}
TRAFFIC_SOURCE = {("crystal_array", 1): "ncu DRAM bytes of k_simulate on a 1M-photon crystal event (an earlier "
                                        "build of that kernel), scaled by photons",
                  ("crystal_array", 2): "ncu DRAM bytes of k_generate + k_simulate_pool on a 2.5M-photon crystal "
                                        "event (commit d060c5a), scaled by photons",
                  ("large_sphere", 3): "ncu DRAM bytes of k_generate + the wavefront passes on a 5M-photon event of "
                                       "the 20,000-sensor sphere (commit 246e140), scaled by photons"}


def pinned_photons(n):
    """A host array of at least n photon records in page-locked memory (the destination of the end-to-end hit
    download), one buffer for the whole run that grows when a larger event needs it (page-locked memory is a limited
    resource: a buffer per configuration had left the later, larger ones pageable); pageable memory if the allocator
    cannot pin it.  pinned_photons.pinned tells which."""
    import torch
    from eic_opticks_gb300 import engine as E
    if pinned_photons.buf is None or pinned_photons.buf.numel() < n * E.L.PHOTON.itemsize:
        pinned_photons.buf = None               # release the smaller buffer before pinning the larger one
        try:
            pinned_photons.buf = torch.empty(n * E.L.PHOTON.itemsize, dtype=torch.uint8, pin_memory=True)
            pinned_photons.pinned = bool(pinned_photons.buf.is_pinned())
        except RuntimeError:
            pinned_photons.pinned = False
            return np.zeros(n, dtype=E.L.PHOTON)
    return pinned_photons.buf.numpy().view(E.L.PHOTON)


pinned_photons.buf = None
pinned_photons.pinned = False


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return float(m["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 50 ms during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), "bench_clocks_%d.csv" % os.getpid())

    def __enter__(self):
        if self.device < 0:          # no sampling asked
            return self
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        try:
            os.remove(self.path)
        except OSError:
            pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


KERNEL_MODES = {0: "photon pool", 1: "one thread per photon", 2: "photon pool over pregenerated photons",
                3: "wavefront (per-step passes over pregenerated photons)"}
KERNEL_NAMES = {0: "k_simulate_pool", 1: "k_simulate", 2: "k_generate + k_simulate_pool",
                3: "k_generate + k_wf_start + k_wf_trace + k_wf_step"}

WORKLOADS = {
    "nested_boxes": "nested_boxes_torch_100k_input_photons",
    "crystal_array": WORKLOAD,
    "water_cube": "water_cube_cerenkov_1000gs",
    "large_sphere": "large_sphere_20000_sensors_scint_100M",
}


def workload(seed=1, num_gs=None, kind="crystal_array"):
    """One event of each benchmark configuration: (geometry arrays, gensteps, input photons or None).

    nested_boxes : 100,000 input photons at the origin, isotropic, 420 nm, in the vacuum/lead/air/water boxes.
    crystal_array: num_gs Poisson(5000) scintillation gensteps in the 8x8 CsI array (the headline event).
    water_cube   : 1,000 Frank-Tamm Cerenkov steps (2 mm, beta 0.8-1) in the 1 m dispersive water cube.
    large_sphere : 20,000 gensteps of 5,000 photons (100M) uniform in r < 17 m of the 17.7 m liquid-scintillator
                   sphere with 20,000 instanced CSG sensors."""
    ge.load_package()
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    if kind == "nested_boxes":
        inp = GS.isotropic_photons(100_000, seed=seed)
        return G.nested_boxes().arrays(), GS.input_photon_genstep(len(inp)), inp
    if kind == "water_cube":
        g = G.water_cube()
        return g.arrays(), GS.water_cerenkov_gensteps(g, 1000, seed=seed), None
    if kind == "large_sphere":
        return G.large_sphere().arrays(), GS.sphere_scint_gensteps(num_gs or 20000, 5000, seed=seed), None
    return G.crystal_array().arrays(), GS.crystal_scint_gensteps(num_gs or 2000, 5000, seed=seed), None


def photon_sample(gs, inp, n):
    """The first n photons of an event: leading gensteps, the last one cut short (input photons sliced alike)."""
    counts = gs.view(np.uint32)[:, 0, 3].astype(np.int64)
    end = np.cumsum(counts)
    k = int(np.searchsorted(end, n))
    if k >= len(gs):
        return gs, inp, int(end[-1]) if len(end) else 0
    sample = gs[:k + 1].copy()
    sample.view(np.uint32)[k, 0, 3] = n - (int(end[k - 1]) if k > 0 else 0)
    return sample, (inp[:n] if inp is not None else None), n


def cpu_baseline(geom, gs, target_s=12.0, threads=None, inp=None):
    """The oracle on a bounded sample (the first photons of the event) using all host cores: the sample grows
    from 256 photons until one timed run takes about a quarter of target_s."""
    O = ge.load_oracle()
    O.build()
    cfg = O.SimConfig(geom)
    threads = threads or os.cpu_count() or 1
    total = int(gs.view(np.uint32)[:, 0, 3].astype(np.int64).sum())
    want = min(256, total)
    while True:
        sample, sinp, n = photon_sample(gs, inp, want)
        t0 = time.perf_counter()
        out, _ = O.simulate(cfg, sample, input_photon=sinp, nthreads=threads, seq=False)
        dt = time.perf_counter() - t0
        if dt > target_s / 4 or n >= total:
            break
        want = min(total, max(want + 1, int(want * target_s / 4 / max(dt, 1e-3))))
    return {"value": n / dt, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": "first %d of %d photons of the event, %.1f s" % (n, total, dt)}


def reference_arm(args):
    """--impl reference : the reference's CPU implementation of the path on the host cores.

    oracle/_ref/libref.so (the reference's own headers compiled for the host) when it was built on this machine,
    else the oracle port.  Each step simulates the next `threads` gensteps of the crystal-array event, one genstep
    per host thread, each with its event photon offset, so the photons are exactly those of the full event."""
    from concurrent.futures import ThreadPoolExecutor
    geom, gs, _ = workload()
    O = ge.load_oracle()
    O.build()
    use_ref = O.reflib() is not None
    kind = "reference" if use_ref else "port"
    cfg = O.SimConfig(geom)
    threads = os.cpu_count() or 1
    counts = gs.view(np.uint32)[:, 0, 3].astype(np.int64)
    begin = np.concatenate([[0], np.cumsum(counts)])
    sample_gs = threads
    times, photons = [], 0

    def one(k):
        out, _ = O.simulate(cfg, gs[k:k + 1], photon_offset=int(begin[k]), seq=False, use_ref=use_ref)
        return len(out)

    with ThreadPoolExecutor(max_workers=threads) as pool:
        for step in range(args.warmup + args.steps):
            first = step * sample_gs % len(gs)
            ks = [(first + j) % len(gs) for j in range(sample_gs)]
            t0 = time.perf_counter()
            n = sum(pool.map(one, ks))
            dt = time.perf_counter() - t0
            if step >= args.warmup:
                times.append(dt)
                photons += n
    total = sum(times)
    value = photons / total
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / max(1, len(times)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample_gensteps_per_step": sample_gs,
                       "sample": "per-photon rate on a bounded sample of the same event: each step simulates %d of its "
                                 "%d gensteps (one per host thread, each with its event photon offset), so the photons "
                                 "are exactly the event's own" % (sample_gs, len(gs))},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                             "sample": "%d gensteps per step, one per thread (~%d photons)"
                                       % (sample_gs, photons // max(1, len(times)))},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def mixed_events(num_events, seed=11, lo=3.0, hi=7.0):
    """Serving workload: events drawn 50/50 from the crystal-array scintillation and water Cerenkov generators,
    photons per event log-uniform in [10^lo, 10^hi]."""
    ge.load_package()
    from eic_opticks_gb300 import geometry as G, gensteps as GS
    rng = np.random.default_rng(seed)
    wc = G.water_cube()
    ca = G.crystal_array()
    events = []
    for k in range(num_events):
        photons = int(10 ** rng.uniform(lo, hi))
        if rng.uniform() < 0.5:
            gs = GS.crystal_scint_gensteps(max(1, photons // 5000), min(5000, photons), seed=5000 + k)
            events.append(("crystal", 10000 + k, gs))
        else:
            gs = GS.water_cerenkov_gensteps(wc, max(1, photons // 100), seed=7000 + k)
            events.append(("water", 10000 + k, gs))
    return {"crystal": ca.arrays(), "water": wc.arrays()}, events


def pct(v, q):
    return float(np.percentile(np.asarray(v), q)) if len(v) else None


def serving_bench(num_events=400, submitters=16, load=0.8, lo=3.0, hi=7.0):
    """Plain one-launch-per-event path vs the continuous-batching server on the mixed serving workload.

    * plain capacity: events processed one synchronous gbo_simulate call at a time (the reference's way);
    * batched capacity: every event submitted at once from `submitters` threads, server drains them;
    * latency under load: Poisson arrivals at `load` x the plain capacity, from `submitters` threads, for both
      paths (the plain path serves arrivals first-come first-served with one call at a time).
    """
    import threading
    from eic_opticks_gb300 import engine as E
    arrays, events = mixed_events(num_events, lo=lo, hi=hi)
    engines = {k: E.Engine(a) for k, a in arrays.items()}
    # kernel form of each engine picked by the autotuner on a sample event of its kind (setup)
    tuned = {}
    for kind, eng in engines.items():
        from eic_opticks_gb300 import geometry as G, gensteps as GS
        sample = (GS.crystal_scint_gensteps(200, 5000, seed=99) if kind == "crystal" else
                  GS.water_cerenkov_gensteps(G.water_cube(), 2000, seed=99))
        r = eng.autotune(0, sample, trials=2)
        tuned[kind] = {"mode": KERNEL_MODES[r["kernel_mode"]], "refill_min": r["refill_min"],
                       "refill_period": r["refill_period"], "blocks_per_sm": r["blocks_per_sm"],
                       "walk_min": r["walk_min"], "rng_call": r["rng_call"]}
    photons = {id(ev[2]): int(ev[2].view(np.uint32)[:, 0, 3].astype(np.int64).sum()) for ev in events}
    total_photons = sum(photons.values())
    for kind, eid, gs in events[:4]:                          # warm-up
        engines[kind].simulate(eid, gs)
    # ---- plain capacity (closed loop), each event's own time kept for the bound below
    event_s = []
    t0 = time.perf_counter()
    for kind, eid, gs in events:
        a = time.perf_counter()
        engines[kind].simulate(eid, gs)
        engines[kind].hits()
        event_s.append(time.perf_counter() - a)
    plain_s = time.perf_counter() - t0
    plain_rate = total_photons / plain_s
    # Photon-weighted upper bound of batched / plain: batching can at best run every photon at the rate the largest
    # events of its kind reach alone, so the stream takes at least sum(photons / peak rate).  It holds only where the
    # largest events fill the GPU (at least the server's target batch of 4M photons); below that, packing events
    # raises the rate beyond any single event's and there is no such bound.
    peak = {}
    for (kind, _, gs), s in zip(events, event_s):
        peak[kind] = max(peak.get(kind, 0.0), photons[id(gs)] / s)
    fills = max(photons.values()) >= (4 << 20)
    bound = plain_s / sum(photons[id(gs)] / peak[kind] for kind, _, gs in events) if fills else None
    servers = {k: E.Server(e, slots=2) for k, e in engines.items()}

    def run_batched(arrivals):
        tickets = [None] * len(events)
        start = time.perf_counter()

        def producer(idx):
            for i in idx:
                if arrivals is not None:
                    delay = start + arrivals[i] - time.perf_counter()
                    if delay > 0:
                        time.sleep(delay)
                kind, eid, gs = events[i]
                tickets[i] = (kind, servers[kind].submit(eid, gs))

        th = [threading.Thread(target=producer, args=(range(j, len(events), submitters),)) for j in range(submitters)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        lat = []
        for kind, t in tickets:
            servers[kind].wait(t)
        elapsed = time.perf_counter() - start
        for kind, t in tickets:
            lat.append(servers[kind].info(t)["latency_s"])
            servers[kind].release(t)
        return elapsed, lat

    run_batched(None)                                       # warm-up of the server buffers
    batched_s, _ = run_batched(None)
    batched_rate = total_photons / batched_s
    # the same drain with each batch's copies and kernels issued one by one instead of as one CUDA graph
    graph_stats = {k: s.stats() for k, s in servers.items()}
    for s in servers.values():
        s.close()
    servers = {k: E.Server(e, slots=2, use_graph=0) for k, e in engines.items()}
    run_batched(None)
    direct_s, _ = run_batched(None)
    for s in servers.values():
        s.close()
    servers = {k: E.Server(e, slots=2) for k, e in engines.items()}
    run_batched(None)
    # ---- latency at `load` x plain capacity, Poisson arrivals
    mean_photons = total_photons / len(events)
    rate_events = load * plain_rate / mean_photons
    rng = np.random.default_rng(3)
    arrivals = np.cumsum(rng.exponential(1.0 / rate_events, len(events)))
    _, lat_b = run_batched(arrivals)
    # plain path on the same arrivals: one call at a time, first come first served
    lat_p = []
    start = time.perf_counter()
    for i in np.argsort(arrivals):
        kind, eid, gs = events[i]
        now = time.perf_counter() - start
        if now < arrivals[i]:
            time.sleep(arrivals[i] - now)
        engines[kind].simulate(eid, gs)
        engines[kind].hits()
        lat_p.append(time.perf_counter() - start - arrivals[i])
    stats = {k: s.stats() for k, s in servers.items()}
    for s in servers.values():
        s.close()
    for e in engines.values():
        e.close()
    return {
        "workload": "mixed 50/50 crystal-array scintillation / water Cerenkov, photons per event log-uniform "
                    "1e%g-1e%g" % (lo, hi),
        "events": len(events), "photons": total_photons, "submitter_threads": submitters,
        "plain_photons_per_s": plain_rate, "batched_photons_per_s": batched_rate,
        "batched_over_plain": batched_rate / plain_rate,
        "batched_over_plain_bound": bound,
        "bound_rule": "plain time / sum over events of photons / (rate of the fastest plain event of its kind)",
        "peak_photons_per_s": peak,
        "batched_without_graph_photons_per_s": total_photons / direct_s,
        "graph": {k: {"launches": v["graph_launches"], "instantiations": v["graph_instantiations"]}
                  for k, v in graph_stats.items()},
        "arrivals": "Poisson at %.0f%% of plain capacity (%.1f events/s)" % (100 * load, rate_events),
        "batched_latency_ms": {"p50": 1e3 * pct(lat_b, 50), "p99": 1e3 * pct(lat_b, 99)},
        "plain_latency_ms": {"p50": 1e3 * pct(lat_p, 50), "p99": 1e3 * pct(lat_p, 99)},
        "batches": {k: v["batches"] for k, v in stats.items()},
        "kernel": tuned,
        "server": {"slots": 2, "target_batch_photon": 4 << 20, "min_batch_photon": 2 << 20, "max_wait_us": 1000,
                   "hbm_budget_bytes": 120 << 30},
    }


def same_config_batching(geom, kind, n_events, tune, submitters=16):
    """n_events events of one configuration (seeds differ): one synchronous gbo_simulate + hit download per event,
    against the server draining all of them submitted at once (continuous batching, graph mode)."""
    import threading
    from eic_opticks_gb300 import engine as E
    events = [workload(seed=100 + k, kind=kind)[1:] for k in range(n_events)]
    photons = sum(int(g.view(np.uint32)[:, 0, 3].astype(np.int64).sum()) for g, _ in events)
    eng = E.Engine(geom, kernel_mode=tune["kernel_mode"], refill_min=tune["refill_min"],
                   refill_period=tune["refill_period"], blocks_per_sm=tune.get("blocks_per_sm", 0),
                   walk_min=tune.get("walk_min", 1), rng_call=tune.get("rng_call", 0))
    eng.simulate(0, *events[0])
    t0 = time.perf_counter()
    for k, (g, inp) in enumerate(events):
        eng.simulate(500 + k, g, inp)
        eng.hits()
    plain_s = time.perf_counter() - t0
    srv = E.Server(eng, slots=2)

    def drain():
        tickets = [None] * n_events
        start = time.perf_counter()

        def producer(idx):
            for i in idx:
                tickets[i] = srv.submit(500 + i, *events[i])

        th = [threading.Thread(target=producer, args=(range(j, n_events, submitters),)) for j in range(submitters)]
        for t in th:
            t.start()
        for t in th:
            t.join()
        for t in tickets:
            srv.wait(t)
        el = time.perf_counter() - start
        lat = []
        for t in tickets:
            lat.append(srv.info(t)["latency_s"])
            srv.release(t)
        return el, lat

    drain()
    batched_s, lat = drain()
    st = srv.stats()
    srv.close()
    eng.close()
    return {"events": n_events, "photons": photons, "plain_photons_per_s": photons / plain_s,
            "batched_photons_per_s": photons / batched_s, "batched_over_plain": plain_s / batched_s,
            "batches": st["batches"], "drain_latency_ms": {"p50": 1e3 * pct(lat, 50), "p99": 1e3 * pct(lat, 99)}}

def measure_workload(kind, args, dist, rank, world, local, steps, warmup, form=None, num_gs=None, precision=0,
                     clocks=False):
    """One configuration on this rank's GPU: device-resident photons/s (value) and photons/s through the C ABI
    with host buffers (e2e), the simulate kernels' algorithmic HBM bytes against the measured copy bandwidth, the
    kernel form the autotuner picked on a 10 % sample.  Returns a dict; the engine and inputs ride along under
    keys starting with '_' for the caller."""
    import torch
    from eic_opticks_gb300 import engine as E
    geom, gs, inp = workload(seed=1 + rank, num_gs=num_gs, kind=kind)
    n_photon = int(gs.view(np.uint32)[:, 0, 3].astype(np.int64).sum())
    n_inp = 0 if inp is None else len(inp)
    if form:
        mode, refill, period, blocks, walk, rcall = (tuple(form) + (0, 1, 0)[len(form) - 3:])[:6]
        eng = E.Engine(geom, device=local, precision=precision, kernel_mode=mode, refill_min=refill,
                       refill_period=period, blocks_per_sm=blocks, walk_min=walk, rng_call=rcall)
        tune = {"kernel_mode": mode, "refill_min": refill, "refill_period": period, "blocks_per_sm": blocks,
                "walk_min": walk, "rng_call": rcall}
    else:
        # kernel form picked by the autotuner on a 10% sample of the workload (setup, outside the timed region)
        eng = E.Engine(geom, device=local, precision=precision)
        if inp is None:
            tune = eng.autotune(0, gs[: max(1, len(gs) // 10)], trials=2)
        else:
            tune = eng.autotune(0, gs, inp, trials=2)

    d_gs = torch.from_numpy(gs.copy()).to(f"cuda:{local}")
    d_inp = torch.from_numpy(inp.view(np.uint8).copy()).to(f"cuda:{local}") if inp is not None else None
    inp_ptr = d_inp.data_ptr() if d_inp is not None else 0
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=f"cuda:{local}")
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    # ---- device-resident throughput (value) ----
    for w in range(warmup):
        eng.simulate_device(w, d_gs.data_ptr(), len(gs), inp_ptr, n_inp)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    ms, sim_ms, gen_ms, launches, hits = [], [], [], 0, 0
    with ClockSampler(local if clocks else -1) as clk:
        for k in range(steps):
            flush.zero_()
            torch.cuda.synchronize()
            start.record()
            hits = eng.simulate_device(1000 + k, d_gs.data_ptr(), len(gs), inp_ptr, n_inp)
            end.record()
            end.synchronize()
            ms.append(start.elapsed_time(end))
            st = eng.stats()
            sim_ms.append(st["ms_simulate"])
            gen_ms.append(st["ms_generate"])
            launches += st["kernel_launches"]
    torch.cuda.synchronize()
    total_ms = sum(ms)
    if dist:
        t = torch.tensor([total_ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t[0])
    value = world * n_photon * steps / (total_ms * 1e-3)

    # ---- end to end through the C ABI with host buffers (e2e) ----
    # one page-locked destination for the whole run, sized from the device-resident events' hit count (events of
    # other ids differ by a few hits); allocated before the timed steps
    hits_host = pinned_photons(int(hits * 1.25) + 4096)
    h2d = gs.nbytes + (inp.nbytes if inp is not None else 0)

    def e2e_steps(run):
        out_ms, nh = [], 0
        for k in range(warmup + steps):
            flush.zero_()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            nh = run(k)
            t1 = time.perf_counter()
            if k >= warmup:
                out_ms.append((t1 - t0) * 1e3)
        total = sum(out_ms)
        if dist:
            t = torch.tensor([total], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            total = float(t[0])
        return world * n_photon * steps / (total * 1e-3), out_ms, nh

    # gbo_simulate_to_host: the call a user makes, hits landing in host memory when it returns
    e2e_value, e2e_ms, nh = e2e_steps(lambda k: eng.simulate_to_host(2000 + k, gs, hits_host, inp))
    launches_e2e = eng.stats()["simulate_launches"]
    # gbo_simulate, then gbo_copy_hits (timed apart)
    sim_part, hit_part = [], []

    def two_calls(k):
        t0 = time.perf_counter()
        n = eng.simulate(4000 + k, gs, inp)
        t1 = time.perf_counter()
        if n > len(hits_host):
            raise RuntimeError("%d hits for a buffer of %d" % (n, len(hits_host)))
        eng.hits(out=hits_host[:n])
        sim_part.append((time.perf_counter() - t1, t1 - t0))
        return n
    two_value, _, _ = e2e_steps(two_calls)
    sim_part = sim_part[warmup:]
    d2h = nh * 64 + 32      # ordered hits + the counters read that sizes them

    hbm, peak_kind = peaks()
    f_hit = hits / n_photon
    b_alg = 96.0 / (n_photon / len(gs)) + 4 + 64 + 64 + 64 * f_hit + (64.0 if inp is not None else 0.0)
    sim_mean = float(np.mean(sim_ms))
    traffic_key = (kind, tune["kernel_mode"])
    achieved = b_alg * n_photon / (sim_mean * 1e-3) / 1e9
    return {
        "value": value, "unit": UNIT, "ms_per_step": total_ms / steps, "steps": steps, "warmup": warmup,
        "config": {"precision": "binary64 root polish + accumulators" if precision else "binary32",
                   "photons_per_step": n_photon, "gensteps_per_step": len(gs), "hits_per_step": hits,
                   "kernel": {"mode": KERNEL_MODES[tune["kernel_mode"]], "refill_min": tune["refill_min"],
                              "refill_period": tune["refill_period"], "blocks_per_sm": tune.get("blocks_per_sm", 0),
                              "walk_min": tune.get("walk_min", 1), "rng_call": tune.get("rng_call", 0),
                              "chosen_by": "--form" if form else "autotuner on 10% sample"},
                   "max_bounce": 31},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "call": "gbo_simulate_to_host", "ms_per_step": float(np.mean(e2e_ms)), "launches": launches_e2e,
                "hit_buffer": "page-locked" if pinned_photons.pinned else "pageable",
                "two_calls": {"value": two_value, "call": "gbo_simulate + gbo_copy_hits",
                              "simulate_ms": float(np.mean([b for _, b in sim_part])),
                              "hit_download_ms": float(np.mean([a for a, _ in sim_part]))}},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": (TRAFFIC_B_PER_PHOTON[traffic_key] * n_photon
                                 if traffic_key in TRAFFIC_B_PER_PHOTON and not precision else None),
                     "traffic_source": (TRAFFIC_SOURCE[traffic_key]
                                        if traffic_key in TRAFFIC_B_PER_PHOTON and not precision else None),
                     "kernel": KERNEL_NAMES[tune["kernel_mode"]], "bytes_per_photon": b_alg,
                     "kernel_ms": sim_mean, "generate_ms": float(np.mean(gen_ms)), "peak_source": peak_kind},
        "clocks": clk.summary() if clocks else None,
        "_engine": eng, "_geom": geom, "_gs": gs, "_inp": inp, "_tune": tune,
    }


def fp64_error_sample(n=100_000, seed=5):
    """Intersection distances of the 20,000-sensor geometry against the binary64 oracle (oracle/orc_csg64.c) on
    n rays (half from inside r < 17 m, half from the water aimed at the sensors), binary32 and precision mode:
    the largest |t - t64| in mm over rays whose closest boundary agrees."""
    from eic_opticks_gb300 import engine as E, geometry as G
    O = ge.load_oracle()
    O.build()
    arrays = G.large_sphere().arrays()
    rng = np.random.default_rng(seed)
    h = n // 2
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = np.concatenate([17000.0 * rng.uniform(0, 1, h) ** (1.0 / 3.0), rng.uniform(17900.0, 18900.0, n - h)])
    pos = r[:, None] * u
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    aim = 19400.0 * u[h:] + rng.normal(scale=300.0, size=(n - h, 3))
    a = aim - pos[h:]
    d[h:] = a / np.linalg.norm(a, axis=1, keepdims=True)
    pos, d = pos.astype(np.float32), d.astype(np.float32)
    t0 = time.perf_counter()
    t64, b64 = O.trace64(O.SimConfig(arrays), pos, d)
    out = {"rays": n, "oracle": "binary64 restatement of the CSG intersection (orc_csg64.c)",
           "oracle_s": time.perf_counter() - t0}
    for precision in (0, 1):
        eng = E.Engine(arrays, precision=precision)
        t, b = eng.trace_rays(pos, d)
        eng.close()
        ok = (b == b64) & (t64 > 0) & (t > 0)
        err = np.abs(t[ok].astype(np.float64) - t64[ok])
        out["binary32" if precision == 0 else "precision_mode"] = {
            "same_boundary": float(ok.mean()), "max_mm": float(err.max()),
            "p99_99_mm": float(np.percentile(err, 99.99)), "above_1e-3_mm": float((err > 1e-3).mean())}
    return out


def other_configs(args, dist, rank, world, local):
    """The remaining benchmark configurations on this GPU, each with its own device-resident and end-to-end
    photons/s, roofline and CPU baseline: nested boxes (100k input photons), dispersive water Cerenkov (1,000
    steps), the 17.7 m sphere with 20,000 instanced sensors (100M photons) in binary32 and in the precision mode,
    with the precision mode's FP64 intersection error on a ray sample."""
    out = {}
    for kind, steps, warmup in (("nested_boxes", 50, 5), ("water_cube", 50, 5), ("large_sphere", 3, 3)):
        m = measure_workload(kind, args, dist, rank, world, local, steps, warmup)
        eng, geom, gs, inp = m.pop("_engine"), m.pop("_geom"), m.pop("_gs"), m.pop("_inp")
        m.pop("_tune")
        eng.close()
        m.pop("clocks")
        m["workload"] = WORKLOADS[kind]
        if not args.no_cpu_baseline:
            m["cpu_baseline"] = cpu_baseline(geom, gs, target_s=4.0, inp=inp)
        out[kind] = m
    m = measure_workload("large_sphere", args, dist, rank, world, local, 2, 3, precision=1)
    for k in ("_engine",):
        m.pop(k).close()
    for k in ("_geom", "_gs", "_inp", "_tune", "clocks"):
        m.pop(k)
    m["workload"] = WORKLOADS["large_sphere"] + "_precision"
    m["fp64_intersection_error"] = fp64_error_sample()
    out["large_sphere_precision"] = m
    return out


def dist_init(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    if ws <= 1:
        return None, 0, 1
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist, dist.get_rank(), ws


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-serving", action="store_true", help="skip the batched-serving comparison")
    ap.add_argument("--gensteps", type=int, default=None,
                    help="gensteps per event (default: the workload's own, 2000 for the crystal array)")
    ap.add_argument("--workload", default="crystal_array", choices=sorted(WORKLOADS))
    ap.add_argument("--form", default=None,
                    help="kernel form MODE,REFILL,PERIOD[,BLOCKS_PER_SM[,WALK_MIN[,RNG_CALL]]] instead of the "
                         "autotuner's choice (MODE 0: photon pool, 1: one thread per photon, 2: photon pool over "
                         "pregenerated photons, 3: wavefront)")
    ap.add_argument("--batch-events", type=int, default=None,
                    help="events of the workload for the same-configuration plain vs batched comparison")
    ap.add_argument("--precision", type=int, default=0, choices=[0, 1],
                    help="1: binary64 root polish and position/time accumulators")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the figures of the other benchmark configurations (nested boxes, water, large sphere)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank == 0:
            reference_arm(args)
        return

    dist, rank, world = dist_init(args)
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    torch.cuda.set_device(local)
    if rank == 0:
        ge.build()
    if dist:
        dist.barrier()
    ge.load_package()
    from eic_opticks_gb300 import engine as E
    form = tuple(int(x) for x in args.form.split(",")) if args.form else None
    m = measure_workload(args.workload, args, dist, rank, world, local, args.steps, args.warmup, form=form,
                         num_gs=args.gensteps, precision=args.precision, clocks=True)
    eng, geom, gs, inp, tune = m.pop("_engine"), m.pop("_geom"), m.pop("_gs"), m.pop("_inp"), m.pop("_tune")

    if rank != 0:
        if dist:
            dist.barrier()
        eng.close()
        return

    line = {
        "metric": METRIC, "value": m["value"], "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": m["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32" if not args.precision else "f32+f64",
        "data": "synthetic (seeded numpy gensteps with the reference genstep layout)",
        "config": dict(m["config"], workload=(WORKLOADS[args.workload] if args.gensteps is None
                                              else WORKLOADS[args.workload] + "_%dgs" % args.gensteps),
                       path="plain: one event per launch", l2="flushed (256 MB write) between timed steps",
                       parallelism="replicas" if world > 1 else "1 GPU"),
        "e2e": m["e2e"], "gpu_launches": m["gpu_launches"], "roofline": m["roofline"], "clocks": m["clocks"],
    }
    if not args.no_serving and world == 1:
        line["serving"] = serving_bench(num_events=400)                     # the 1e3-1e7 serving stream
        line["serving_small_events"] = serving_bench(num_events=1500, lo=3.0, hi=5.0)
    n_batch = args.batch_events if args.batch_events is not None else (
        {"nested_boxes": 64, "water_cube": 16, "crystal_array": 8, "large_sphere": 2}[args.workload])
    if n_batch > 0 and world == 1 and not args.precision:
        line["same_config_batching"] = same_config_batching(geom, args.workload, n_batch, tune)
    # hit merge (identity, 1 ns bucket) of the last event's hits, as the reference's per-launch merge does
    import ctypes as C
    nm = C.c_int64()
    eng.simulate(3000, gs, inp)
    E._check(eng.lib.gbo_merge_hits(eng.handle, C.c_float(1.0), C.byref(nm)), "gbo_merge_hits")    # warm-up
    t0 = time.perf_counter()
    E._check(eng.lib.gbo_merge_hits(eng.handle, C.c_float(1.0), C.byref(nm)), "gbo_merge_hits")
    line["hit_merge"] = {"time_window_ns": 1.0, "hits": eng.num_hit(), "merged": nm.value,
                         "ms": 1e3 * (time.perf_counter() - t0)}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(geom, gs, inp=inp)
    if not args.no_configs and world == 1 and args.gensteps is None and not args.precision:
        line["configs"] = other_configs(args, dist, rank, world, local)
    print(json.dumps(line))
    if dist:
        dist.barrier()
    eng.close()


if __name__ == "__main__":
    main()
