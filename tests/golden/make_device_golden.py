"""Reference-device fixtures: the reference's own hot-path headers compiled by nvcc for sm_103a
(oracle/ref_device.cu) and run on the GPU, one thread per photon, over

* the inputs of every host fixture (tests/golden/sim_*.npz)  -> dev_<name>.npz  (photons and flag histories);
* 100k-photon samples of the benchmark configurations          -> dev_cfg*.npz
  (1: nested boxes, 100,000 isotropic input photons; 2: the first 100,000 photons of the 2,000-genstep crystal
  event; 3: the whole 1,000-genstep water Cerenkov event; 5: the first 100,000 photons of the 100M-photon event in
  the 17.7 m sphere with its 20,000 instanced CSG sensors).

The reference tree and the GPU live on different machines, so this runs in two steps:

    GBO_REFERENCE_DIR=<reference checkout> make -C oracle ref-device     # -> oracle/_ref/ref_device.cubin
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
                "gdml_raindrop", "gdml_sipm8x8", "gdml_sphere_leak", "gdml_basic_detector"]
GEOM_KEYS = ("node", "prim", "solid", "inst", "itra", "plan", "bnd", "optical", "icdf")
SAMPLE = 100_000


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).view(np.uint8).tobytes()).hexdigest()


def geometry_digest(arrays):
    h = hashlib.sha256()
    for k in GEOM_KEYS:
        h.update(np.ascontiguousarray(arrays[k]).view(np.uint8).tobytes())
    return h.hexdigest()


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


def main(outdir):
    os.makedirs(outdir, exist_ok=True)
    for name in SIM_FIXTURES:
        z = np.load(os.path.join(HERE, "sim_%s.npz" % name))
        cfg = O.SimConfig(golden_arrays(z))
        inp = z["input_photon"] if len(z["input_photon"]) else None
        t0 = time.time()
        p, s, ms = O.ref_device_simulate(cfg, z["gs"], inp, event_index=int(z["event_index"]))
        host = z["photon"]
        same = np.all(s["seqhis"] == z["seq"]["seqhis"], axis=1).mean() if len(p) else 1.0
        exact = np.all(p.view(np.uint32).reshape(-1, 16) == host.view(np.uint32).reshape(-1, 16), axis=1).mean() \
            if len(p) else 1.0
        print("%s: %d photons, %.1f ms; device vs host reference build: history %.5f, bit-exact records %.5f"
              % (name, len(p), ms, same, exact), flush=True)
        save(outdir, "dev_%s.npz" % name, photon=p, seq=s, kernel_ms=np.float32(ms))
    for name in CONFIGS:
        arrays, gs, inp, ev = config_inputs(name)
        cfg = O.SimConfig(arrays)
        t0 = time.time()
        p, s, ms = O.ref_device_simulate(cfg, gs, inp, event_index=ev)
        print("%s: %d photons, kernel %.1f ms, %.1f s" % (name, len(p), ms, time.time() - t0), flush=True)
        save(outdir, "dev_%s.npz" % name, gs=gs, event_index=np.int32(ev), geometry_sha256=geometry_digest(arrays),
             input_photon_sha256=digest(inp) if inp is not None else "", photon=p, seqhis=s["seqhis"],
             kernel_ms=np.float32(ms))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else HERE)
