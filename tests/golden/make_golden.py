"""Generate the golden fixtures in tests/golden/ from the reference's own code compiled for the host.

Run from the repository root in a checkout where the reference tree is available:

    GBO_REFERENCE_DIR=<reference checkout> make -C oracle ref && python tests/golden/make_golden.py [philox csg sims]

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


def trd_planes(hx1, hy1, hx2, hy2, hz):
    """Outward face planes (nx, ny, nz, d) and box of a trd: half lengths (hx1, hy1) at z = -hz, (hx2, hy2) at +hz."""
    v = np.array([(sx * hx, sy * hy, z) for z, hx, hy in ((-hz, hx1, hy1), (hz, hx2, hy2))
                  for sx in (-1, 1) for sy in (-1, 1)], dtype=np.float64)
    faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
    centre = v.mean(axis=0)
    planes = []
    for f in faces:
        n = np.cross(v[f[1]] - v[f[0]], v[f[2]] - v[f[0]])
        n /= np.linalg.norm(n)
        if np.dot(n, v[f[0]] - centre) < 0:
            n = -n
        planes.append((*n, float(np.dot(n, v[f[0]]))))
    return planes, (*v.min(axis=0), *v.max(axis=0))


def csg_shapes():
    """The CSG shapes of csg.npz, each a prim to intersect in its own frame."""
    trd, trd_box = trd_planes(60.0, 50.0, 30.0, 20.0, 80.0)
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
        # added after the shapes above so that their rays stay the same
        "convexpolyhedron": G.convexpolyhedron(trd, trd_box),
        "contiguous": G.csg_list(L.CSG_CONTIGUOUS, [
            G.box3(150, 150, 150), G.cylinder(60, -160, 160),
            G.with_transform(G.box3(100, 100, 100), G.translate(90, 90, 40))]),
        "discontiguous": G.csg_list(L.CSG_DISCONTIGUOUS, [
            G.with_transform(G.sphere(70), G.translate(-120, 0, 0)),
            G.with_transform(G.box3(100, 100, 100), G.translate(120, 0, 0)),
            G.with_transform(G.cylinder(50, -50, 50), G.translate(0, 130, 0))]),
        "overlap": G.csg_list(L.CSG_OVERLAP, [G.sphere(120), G.box3(180, 180, 180), G.cylinder(100, -200, 200)]),
        "difference_list": G.operation(L.CSG_DIFFERENCE, G.box3(240, 240, 240), G.csg_list(L.CSG_DISCONTIGUOUS, [
            G.with_transform(G.cylinder(30, -130, 130), G.translate(-60, 0, 0)),
            G.with_transform(G.cylinder(30, -130, 130), G.translate(60, 0, 0))])),
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
        plan = a["plan"] if len(a["plan"]) else np.zeros((1, 4), np.float32)
        for i in range(n):
            v, r = O.intersect_prim(a["node"], plan, itra, 0.05, o[i], d[i], use_ref=True)
            valid[i] = v
            res[i] = r
        out[name + "_node"] = a["node"]
        out[name + "_itra"] = itra
        out[name + "_plan"] = plan
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


def lists_geometry():
    """A geometry of the list and polyhedron shapes of csg_shapes(), each a glass instance in a vacuum box: the
    multi-union carries a sensor surface, the trd a polished surface, the others plain glass."""
    shapes = csg_shapes()
    g = G.Geometry("csg_lists")
    vac = G.Material("Vacuum", rindex=1.0)
    glass = G.Material("Glass", rindex=1.5, abslength=2e3)
    b_world = g.boundary(vac, None, None, vac)
    b_sensor = g.boundary(vac, G.Surface.sensor("ListSensor", 0.5), None, glass)
    b_mirror = g.boundary(vac, G.Surface.polished("TrdMirror", 0.9), None, glass)
    b_glass = g.boundary(vac, None, None, glass)
    s_world = g.add_solid("world", [(G.box3(1400, 1400, 1400), b_world)])
    placed = [("contiguous", b_sensor, (-320, 0, 0)), ("convexpolyhedron", b_mirror, (320, 0, 0)),
              ("overlap", b_glass, (0, 320, 0)), ("difference_list", b_glass, (0, -320, 0)),
              ("discontiguous", b_glass, (0, 0, 320))]
    g.add_instance(s_world)
    for k, (name, bnd, at) in enumerate(placed):
        s = g.add_solid(name[:15], [(shapes[name], bnd)])
        g.add_instance(s, G.translate(*at), sensor_identifier=k if name == "contiguous" else -1,
                       sensor_index=k if name == "contiguous" else -1)
    g.icdf = G.default_icdf()
    return g


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


def sims_lists():
    gsl = np.concatenate([GS.torch_gensteps(1, 1000, torch_type=t, pos=(0, 0, 0), radius=10.0)
                          for t in (L.T_SPHERE, L.T_SPHERE_MARSAGLIA)])
    sim_case("csg_lists", lists_geometry(), gsl, event_index=1)


if __name__ == "__main__":
    what = sys.argv[1:] or ["philox", "csg", "sims"]
    if "philox" in what:
        philox()
    if "csg" in what:
        csg()
    if "sims" in what:
        sims()
    if "sims" in what or "lists" in what:
        sims_lists()
