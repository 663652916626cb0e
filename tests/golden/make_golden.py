"""Generate the golden fixtures in tests/golden/ from the reference's own code compiled for the host.

Run from the repository root in a checkout where the reference tree is available:

    make -C oracle ref && python tests/golden/make_golden.py

The fixtures are outputs of oracle/_ref/libref.so, which compiles the reference's qsim.h / csg_intersect_*.h
headers unmodified and calls curand's own host Philox.  Each fixture stores its inputs (geometry arrays,
gensteps, rays) next to the reference outputs so that the tests can replay them without the reference tree.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

ge.load_package()
O = ge.load_oracle()
from eic_opticks_gb300 import geometry as G, gensteps as GS, layout as L  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
GEOM_KEYS = ("node", "prim", "solid", "inst", "itra", "plan", "bnd", "optical", "icdf")


def save(name, **kw):
    path = os.path.join(HERE, name)
    np.savez_compressed(path, **kw)
    print("wrote", path, os.path.getsize(path))


def philox():
    cases = np.array([(0, 0, 0, 0), (0, 5, 0, 0), (0, 123456789, 0, 100000), (42, 2**40 + 5, 1, 5),
                      (7, 99, 2, 3), (0, 2**33 - 1, 0, 100000 * 31), (0xDEADBEEFCAFE, 17, 3, 0)], dtype=np.uint64)
    out = np.stack([O.philox_uniforms(int(s), int(q), int(o), int(k), 64, use_ref=True) for s, q, o, k in cases])
    save("philox.npz", cases=cases, uniforms=out)


def csg_shapes():
    """The CSG shapes of csg.npz, each a prim to intersect in its own frame."""
    return {
        "sphere": G.sphere(100), "zsphere": G.zsphere(100, -30, 60), "cylinder": G.cylinder(50, -80, 80),
        "cone": G.cone(80, -50, 20, 70), "box3": G.box3(50, 80, 120),
        "hyperboloid": G._node(L.CSG_HYPERBOLOID, (40, 60, -100, 100), bbox=(-100, -100, -100, 100, 100, 100)),
        "halfspace": G._node(L.CSG_HALFSPACE, (0.3, 0.4, float(np.sqrt(0.75)), 10.0), bbox=(-1e3,) * 3 + (1e3,) * 3),
        "phicut": G._node(L.CSG_PHICUT, (1, 0, 0, 1), bbox=(-1e3,) * 3 + (1e3,) * 3),
        "ellipsoid": G.with_transform(G.sphere(100), G.scale(1, 1, 0.5)),
        "difference": G.operation(L.CSG_DIFFERENCE, G.box3(150, 150, 150), G.sphere(90)),
        "intersection": G.operation(L.CSG_INTERSECTION, G.box3(150, 150, 150), G.sphere(90)),
        "union3": G.operation(L.CSG_UNION, G.operation(L.CSG_UNION, G.with_transform(G.sphere(254), G.scale(1, 1, 184 / 254)),
                                                       G.with_transform(G.cylinder(127, -100, 100), G.translate(0, 0, -184))),
                              G.with_transform(G.cylinder(50, -30, 30), G.translate(0, 0, -313))),
    }


def csg():
    rng = np.random.default_rng(7)
    shapes = csg_shapes()
    out = {}
    n = 2000
    for name, nd in shapes.items():
        gg = G.Geometry()
        gg.boundary(G.Material("a"), None, None, G.Material("b"))
        gg.add_solid("x", [(nd, 0)])
        a = gg.arrays()
        o = rng.uniform(-250, 250, (n, 3)).astype(np.float32)
        d = rng.normal(size=(n, 3))
        d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        res = np.zeros((n, 4), dtype=np.float32)
        valid = np.zeros(n, dtype=np.int8)
        itra = a["itra"] if len(a["itra"]) else np.zeros((1, 4, 4), np.float32)
        for i in range(n):
            v, r = O.intersect_prim(a["node"], np.zeros((1, 4), np.float32), itra, 0.05, o[i], d[i], use_ref=True)
            valid[i] = v
            res[i] = r
        out[name + "_node"] = a["node"]
        out[name + "_itra"] = itra
        out[name + "_o"] = o
        out[name + "_d"] = d
        out[name + "_isect"] = res
        out[name + "_valid"] = valid
    save("csg.npz", names=np.array(list(shapes.keys())), **out)


def sim_case(name, geom, gs, photons=None, event_index=0):
    arrays = geom.arrays()
    cfg = O.SimConfig(arrays)
    out, seq = O.simulate(cfg, gs, photons, event_index=event_index, use_ref=True)
    kw = {k: arrays[k] for k in GEOM_KEYS}
    kw["hd_factor"] = np.array(arrays["hd_factor"])
    kw["domain"] = np.array(arrays["domain"], dtype=np.float32)
    kw["gs"] = gs
    kw["input_photon"] = photons if photons is not None else np.zeros(0, dtype=L.PHOTON)
    kw["event_index"] = np.array(event_index)
    kw["photon"] = out
    kw["seq"] = seq
    save("sim_%s.npz" % name, **kw)


def sims():
    ph = GS.isotropic_photons(3000)
    sim_case("nested_boxes", G.nested_boxes(), GS.input_photon_genstep(len(ph)), ph)
    ph2 = GS.isotropic_photons(1000, seed=3)
    sim_case("nested_boxes_sensor", G.nested_boxes(sensor=True), GS.input_photon_genstep(len(ph2)), ph2, event_index=3)
    sim_case("crystal_array", G.crystal_array(), GS.crystal_scint_gensteps(16, 150, seed=5))
    wc = G.water_cube()
    sim_case("water_cube", wc, GS.water_cerenkov_gensteps(wc, 30, seed=9))
    gst = np.concatenate([GS.torch_gensteps(1, 60, torch_type=t, pos=(0, 0, 0), radius=30.0)
                          for t in (L.T_DISC, L.T_SPHERE, L.T_SPHERE_MARSAGLIA, L.T_POINT, L.T_CIRCLE, L.T_RECTANGLE)])
    sim_case("torch", G.nested_boxes(), gst)
    ls = G.large_sphere(num_sensors=150, sphere_radius=1770.0, sensor_radius=1940.0, shell=12.0)
    sim_case("large_sphere_small", ls, GS.sphere_scint_gensteps(10, 100, seed=11, radius=1700.0))


if __name__ == "__main__":
    philox()
    csg()
    sims()
