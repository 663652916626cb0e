"""Reference-device fixtures: the reference's own hot-path headers compiled by nvcc for sm_103a
(oracle/ref_device.cu) and run on the GPU, one thread per photon, over

* the inputs of every host fixture (tests/golden/sim_*.npz)  -> dev_<name>.npz  (photons and flag histories);
* 100k-photon samples of the benchmark configurations          -> dev_cfg*.npz
  (1: nested boxes, 100,000 isotropic input photons; 2: the first 100,000 photons of the 2,000-genstep crystal
  event; 3: the whole 1,000-genstep water Cerenkov event; 5: the first 100,000 photons of the 100M-photon event in
  the 17.7 m sphere with its 20,000 instanced CSG sensors).

Two builds of the same reference source are run: nvcc's default (multiply-add contraction on, as the reference's own
CUDA build compiles) and --fmad=false (every binary32 multiply and add rounded on its own).

* dev_<name>.npz       photons and flag histories of the default build, plus how far the --fmad=false build of the
                       same reference source lands from it (the fractions of photons within 1e-3 mm / 1e-3 ns): the
                       reference's own sensitivity to contraction;
* dev_nofma_<name>.npz a 64-bit digest per photon of the --fmad=false build's record and flag history, for the
                       bit-exact comparison with the engine built the same way.

The reference tree and the GPU live on different machines, so this runs in two steps:

    GBO_REFERENCE_DIR=<reference checkout> make -C oracle ref-device     # -> oracle/_ref/ref_device*.cubin
    make -C oracle ref-device-run && python tests/golden/make_device_golden.py <outdir>   # on the GPU machine

and the written files are copied into tests/golden/.  The configuration fixtures store their gensteps and the
SHA-256 of the geometry arrays and input photons they were made from; the tests rebuild those inputs with the
package's generators and refuse to compare if a digest differs.
"""
import hashlib
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

ge.load_package()
O = ge.load_oracle()
from eic_opticks_gb300 import geometry as G, gensteps as GS, layout as L  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
SIM_FIXTURES = ["nested_boxes", "nested_boxes_sensor", "crystal_array", "water_cube", "torch", "large_sphere_small",
                "gdml_raindrop", "gdml_sipm8x8", "gdml_sphere_leak", "gdml_basic_detector", "csg_lists"]
GEOM_KEYS = ("node", "prim", "solid", "inst", "itra", "plan", "bnd", "optical", "icdf")
SAMPLE = 100_000


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def geometry_digest(arrays):
    h = hashlib.sha256()
    for k in GEOM_KEYS:
        h.update(np.ascontiguousarray(arrays[k]).view(np.uint8).tobytes())
    return h.hexdigest()


def record_digest(photon, seqhis):
    """One 64-bit digest per photon of its 64-byte record and its flag history (FNV-1a style over the ten 64-bit
    words): equal digests mean bit-identical photons."""
    w = np.concatenate([np.ascontiguousarray(photon).view(np.uint64).reshape(len(photon), 8),
                        np.ascontiguousarray(seqhis).view(np.uint64).reshape(len(photon), 2)], axis=1)
    d = np.full(len(photon), 0xCBF29CE484222325, dtype=np.uint64)
    prime = np.uint64(0x100000001B3)
    with np.errstate(over="ignore"):
        for k in range(w.shape[1]):
            d = (d ^ w[:, k]) * prime
    return d


def strict_fractions(a, b):
    """Fractions of photons whose positions agree within 1e-3 mm and whose times agree within 1e-3 ns (or one ulp
    of the value where that is larger)."""
    if len(a) == 0:
        return 1.0, 1.0
    pos_ok = np.all(np.abs(a["pos"] - b["pos"]) <= np.maximum(1e-3, np.spacing(np.abs(b["pos"]))), axis=1)
    t_ok = np.abs(a["time"] - b["time"]) <= np.maximum(1e-3, np.spacing(np.abs(b["time"])))
    return float(pos_ok.mean()), float(t_ok.mean())


def first_photons(gs, n):
    """The leading gensteps of an event holding its first n photons, the last one cut short."""
    counts = gs.view(np.uint32)[:, 0, 3].astype(np.int64)
    end = np.cumsum(counts)
    k = int(np.searchsorted(end, n))
    if k >= len(gs):
        return gs.copy()
    sample = gs[:k + 1].copy()
    sample.view(np.uint32)[k, 0, 3] = n - (int(end[k - 1]) if k > 0 else 0)
    return sample


def config_inputs(name):
    """(geometry arrays, gensteps, input photons or None, event index) of one benchmark-configuration sample.
    The tests call this too, so fixtures and tests build identical inputs."""
    if name == "cfg1_nested_boxes":
        inp = GS.isotropic_photons(SAMPLE, seed=1)
        return G.nested_boxes().arrays(), GS.input_photon_genstep(len(inp)), inp, 0
    if name == "cfg2_crystal_array":
        return G.crystal_array().arrays(), first_photons(GS.crystal_scint_gensteps(2000, 5000, seed=1), SAMPLE), None, 1
    if name == "cfg3_water_cube":
        g = G.water_cube()
        return g.arrays(), GS.water_cerenkov_gensteps(g, 1000, seed=1), None, 2
    if name == "cfg5_large_sphere":
        return (G.large_sphere().arrays(), first_photons(GS.sphere_scint_gensteps(20000, 5000, seed=1), SAMPLE),
                None, 3)
    raise KeyError(name)


CONFIGS = ["cfg1_nested_boxes", "cfg2_crystal_array", "cfg3_water_cube", "cfg5_large_sphere"]


def golden_arrays(z):
    a = {k: z[k] for k in GEOM_KEYS}
    a["hd_factor"] = int(z["hd_factor"])
    a["domain"] = tuple(float(x) for x in z["domain"])
    return a


def save(outdir, name, **kw):
    path = os.path.join(outdir, name)
    np.savez_compressed(path, **kw)
    print("wrote %s (%d bytes)" % (path, os.path.getsize(path)), flush=True)


def run_both(cfg, gs, inp, ev, name):
    p, s, ms = O.ref_device_simulate(cfg, gs, inp, event_index=ev)
    q, qs, _ = O.ref_device_simulate(cfg, gs, inp, event_index=ev, variant="nofma")
    self_pos, self_time = strict_fractions(q, p)
    hist = float(np.all(qs["seqhis"] == s["seqhis"], axis=1).mean()) if len(p) else 1.0
    print("%s: %d photons, kernel %.1f ms; contraction off vs on: history %.5f, within 1e-3 mm %.5f, within "
          "1e-3 ns %.5f" % (name, len(p), ms, hist, self_pos, self_time), flush=True)
    extra = dict(self_history=np.float64(hist), self_pos=np.float64(self_pos), self_time=np.float64(self_time),
                 kernel_ms=np.float32(ms))
    return p, s, q, qs, extra


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    for name in SIM_FIXTURES:
        z = np.load(os.path.join(HERE, "sim_%s.npz" % name))
        cfg = O.SimConfig(golden_arrays(z))
        inp = z["input_photon"] if len(z["input_photon"]) else None
        p, s, q, qs, extra = run_both(cfg, z["gs"], inp, int(z["event_index"]), name)
        save(outdir, "dev_%s.npz" % name, photon=p, seq=s, **extra)
        save(outdir, "dev_nofma_%s.npz" % name, digest=record_digest(q, qs["seqhis"]))
    for name in CONFIGS:
        arrays, gs, inp, ev = config_inputs(name)
        cfg = O.SimConfig(arrays)
        p, s, q, qs, extra = run_both(cfg, gs, inp, ev, name)
        save(outdir, "dev_%s.npz" % name, gs=gs, event_index=np.int32(ev), geometry_sha256=geometry_digest(arrays),
             input_photon_sha256=digest(inp) if inp is not None else "", photon=p, seqhis=s["seqhis"], **extra)
        save(outdir, "dev_nofma_%s.npz" % name, digest=record_digest(q, qs["seqhis"]))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
