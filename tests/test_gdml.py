"""GDML loader: the reference's own test geometries and its file-photon pin, and each supported solid and
structure element on a small document of our own."""
import math
import os

import numpy as np
import pytest

from conftest import golden_arrays, load_golden

REF_GEOM = os.path.join(os.environ.get("GBO_REFERENCE_DIR") or os.devnull, "tests", "geom")


def test_raindrop_file_photons_all_hit(oracle):
    """tests/test_GPUPhotonFileSource.sh: the ten file photons in opticks_raindrop.gdml all end as hits with their
    wavelengths unchanged (3 x 420, 2 x 450, 5 x 500 nm)."""
    z = load_golden("sim_gdml_raindrop.npz")
    out, _ = oracle.simulate(oracle.SimConfig(golden_arrays(z)), z["gs"], z["input_photon"])
    hit = (out["flagmask"] & (1 << 6)) != 0
    assert hit.all()
    assert sorted(out["wavelength"][hit].tolist()) == [420.0] * 3 + [450.0] * 2 + [500.0] * 5


@pytest.mark.skipif(not os.path.isdir(REF_GEOM), reason="reference tree not present")
@pytest.mark.parametrize("name,fname", [("raindrop", "opticks_raindrop.gdml"), ("sipm8x8", "8x8SiPM_w_CSI_optial_grease.gdml"),
                                        ("sphere_leak", "sphere_leak.gdml"), ("basic_detector", "basic_detector.gdml")])
def test_loader_reproduces_fixture(name, fname):
    from eic_opticks_gb300 import gdml
    g, _ = gdml.load(os.path.join(REF_GEOM, fname))
    a = g.arrays()
    z = load_golden("sim_gdml_%s.npz" % name)
    for k in ("node", "prim", "inst", "itra", "plan", "bnd", "optical", "icdf"):
        assert np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(z[k]).view(np.uint8)), (name, k)


@pytest.mark.skipif(not os.path.isdir(REF_GEOM), reason="reference tree not present")
def test_loader_reads_every_reference_geometry():
    from eic_opticks_gb300 import gdml
    for f in sorted(os.listdir(REF_GEOM)):
        if f.endswith(".gdml"):
            g, doc = gdml.load(os.path.join(REF_GEOM, f))
            a = g.arrays()
            assert len(a["inst"]) == len(doc.placements) >= 2, f


DOC = """<?xml version="1.0"?>
<gdml>
  <define>
    <constant name="HALF" value="50"/>
    <variable name="k" value="0"/>
    <matrix name="RI_W" coldim="2" values="1.5*eV 1.33 6.2*eV 1.36"/>
    <matrix name="RI_A" coldim="2" values="1.5e-06 1.0 6.2e-06 1.0"/>
    <matrix name="ABS_W" coldim="2" values="1.5*eV 10*m 6.2*eV 10*m"/>
    <matrix name="EFF" coldim="2" values="1.5*eV 0.25 6.2*eV 0.25"/>
    <matrix name="REFL" coldim="2" values="1.5*eV 0.9 6.2*eV 0.9"/>
    <rotation name="r90" x="90" unit="deg"/>
  </define>
  <materials>
    <material name="Air"><property name="RINDEX" ref="RI_A"/></material>
    <material name="Water"><property name="RINDEX" ref="RI_W"/><property name="ABSLENGTH" ref="ABS_W"/></material>
    <material name="Steel"/>
  </materials>
  <solids>
    <box name="World" x="1000" y="1000" z="1000"/>
    <tube name="Pipe" rmin="10" rmax="20" z="2*HALF" deltaphi="360" aunit="deg"/>
    <sphere name="Cap" rmax="30" deltatheta="90" aunit="deg"/>
    <ellipsoid name="Bulb" ax="40" by="40" cz="20" zcut2="10"/>
    <cone name="Cup" rmin1="0" rmax1="20" rmin2="0" rmax2="10" z="40"/>
    <polycone name="Horn" startphi="0" deltaphi="360" aunit="deg">
      <zplane rmin="0" rmax="10" z="-20"/><zplane rmin="0" rmax="10" z="0"/><zplane rmin="0" rmax="25" z="20"/>
    </polycone>
    <trd name="Wedge" x1="40" x2="20" y1="40" y2="20" z="30"/>
    <orb name="Ball" r="5"/>
    <union name="Tee">
      <first ref="Pipe"/><second ref="Pipe"/>
      <position name="tp" x="0" y="0" z="0"/><rotationref ref="r90"/>
    </union>
    <opticalsurface name="Det" model="glisur" finish="polished" type="dielectric_metal" value="1">
      <property name="EFFICIENCY" ref="EFF"/>
    </opticalsurface>
    <opticalsurface name="Mirror" model="glisur" finish="ground" type="dielectric_metal" value="1">
      <property name="REFLECTIVITY" ref="REFL"/>
    </opticalsurface>
  </solids>
  <structure>
    <volume name="BallLV"><materialref ref="Water"/><solidref ref="Ball"/></volume>
    <volume name="TeeLV"><materialref ref="Steel"/><solidref ref="Tee"/></volume>
    <volume name="CapLV"><materialref ref="Water"/><solidref ref="Cap"/></volume>
    <volume name="BulbLV"><materialref ref="Water"/><solidref ref="Bulb"/></volume>
    <volume name="CupLV"><materialref ref="Water"/><solidref ref="Cup"/></volume>
    <volume name="HornLV"><materialref ref="Water"/><solidref ref="Horn"/></volume>
    <volume name="WedgeLV"><materialref ref="Water"/><solidref ref="Wedge"/></volume>
    <volume name="WorldLV">
      <materialref ref="Air"/><solidref ref="World"/>
      <physvol name="tee"><volumeref ref="TeeLV"/><position name="p1" x="-300" y="0" z="0"/></physvol>
      <physvol name="cap"><volumeref ref="CapLV"/><position name="p2" x="0" y="-300" z="0"/></physvol>
      <physvol name="bulb"><volumeref ref="BulbLV"/><position name="p3" x="0" y="300" z="0"/></physvol>
      <physvol name="cup"><volumeref ref="CupLV"/><position name="p4" x="300" y="0" z="0"/>
        <rotation name="r4" y="90" unit="deg"/></physvol>
      <physvol name="horn"><volumeref ref="HornLV"/><position name="p5" x="0" y="0" z="300"/></physvol>
      <physvol name="wedge"><volumeref ref="WedgeLV"/><position name="p6" x="0" y="0" z="-300"/></physvol>
      <loop for="k" from="0" to="2" step="1">
        <physvol name="ball_{k}"><volumeref ref="BallLV"/><position name="pb" x="100*k - 100" y="100" z="100"/></physvol>
      </loop>
    </volume>
    <bordersurface name="DetBS" surfaceproperty="Det"><physvolref ref="cap"/><physvolref ref="WorldLV_PV"/></bordersurface>
    <skinsurface name="MirrorSkin" surfaceproperty="Mirror"><volumeref ref="BulbLV"/></skinsurface>
  </structure>
  <setup name="Default" version="1.0"><world ref="WorldLV"/></setup>
</gdml>
"""


def _trace(oracle, a, o, d):
    cfg = oracle.SimConfig(a)
    t, b = oracle.trace(cfg, np.array([o], np.float32), np.array([d], np.float32), tmin=0.0)
    return float(t[0]), int(b[0])


def test_loader_solids_structure_and_surfaces(oracle):
    from eic_opticks_gb300 import gdml, layout as L
    g, doc = gdml.load(DOC)
    a = g.arrays()
    names = [p[0] for p in doc.placements]
    assert len(names) == 10 and {"ball_0", "ball_1", "ball_2"} <= set(names)          # loop expanded
    # boundaries: Steel has no RINDEX -> implicit absorber osur on Air/Steel; the cap's border surface is the isur
    # of its boundary (cap -> world); the bulb's skin surface is both osur and isur
    bnames = {}
    for pv, lv, b, inst in doc.placements:
        om, os_, is_, im = g.boundaries[b]
        bnames[pv] = (g.materials[om].name, g.surfaces[os_].name if os_ >= 0 else "-",
                      g.surfaces[is_].name if is_ >= 0 else "-", g.materials[im].name)
    assert bnames["tee"][1].startswith("Implicit_RINDEX_NoRINDEX") and bnames["tee"][2] == "-"
    assert bnames["cap"][1:3] == ("-", "DetBS")
    assert bnames["bulb"][1:3] == ("MirrorSkin", "MirrorSkin")
    det = g.surfaces[[s.name for s in g.surfaces].index("DetBS")]
    assert np.allclose(det.detect, 0.25) and np.allclose(det.absorb, 0.75)
    mir = g.surfaces[[s.name for s in g.surfaces].index("MirrorSkin")]
    assert np.allclose(mir.diffuse, 0.9) and np.allclose(mir.specular, 0.0)             # ground -> diffuse
    sens = a["inst"].view(np.int32)[:, 2, 3] > 0
    assert sens.sum() == 1
    # water: RINDEX from eV-tabulated values, ABSLENGTH 10 m in mm
    water = g.materials[[m.name for m in g.materials].index("Water")]
    assert abs(water.abslength[400] - 1e4) < 1e-6 and 1.33 <= water.rindex.min() <= water.rindex.max() <= 1.36
    # geometry by ray: distances in the world frame against the translated CSG
    t, _ = _trace(oracle, a, (0, -300, 100), (0, 0, -1))           # cap: upper hemisphere r 30 at y=-300
    assert abs(t - 70.0) < 1e-3
    t, _ = _trace(oracle, a, (-300, 0, 200), (0, 0, -1))           # tee: down the hollow z pipe's axis, the
    assert abs(t - 180.0) < 1e-3                                   # y pipe's wall (r 10-20) is met at z = 20
    t, _ = _trace(oracle, a, (0, 300, 100), (0, 0, -1))            # bulb: ellipsoid semi-axis z 20, cut at z=10
    assert abs(t - 90.0) < 1e-3
    t, _ = _trace(oracle, a, (400, 0, 0), (-1, 0, 0))              # cup rotated about y: its +z apex faces -x
    assert abs(t - 80.0) < 1e-3                                    # base (r 20) at x = 300 + 20
    t, _ = _trace(oracle, a, (0, 0, 400), (0, 0, -1))              # horn: top at z = 300 + 20
    assert abs(t - 80.0) < 1e-3
    t, _ = _trace(oracle, a, (0, 0, -400), (0, 0, 1))              # wedge: z from -315 to -285
    assert abs(t - 85.0) < 1e-3
    t, _ = _trace(oracle, a, (0, 0, -300), (1, 0, 0))              # wedge mid-plane half width (20 + 10) / 2
    assert abs(t - 15.0) < 1e-3
    assert len(a["plan"]) == 6


def test_expression_evaluator_refuses_code():
    from eic_opticks_gb300 import gdml
    ex = gdml.Expr()
    assert ex("2*pi") == pytest.approx(2 * math.pi) and ex("10*cm") == 100.0 and ex("2^3") == 8.0
    for bad in ("__import__('os')", "open('x')", "(1).__class__", "[1,2]", "lambda: 1"):
        with pytest.raises((ValueError, SyntaxError)):
            ex(bad)


def test_csgfoundry_round_trip(oracle, tmp_path):
    """A CSGFoundry folder in the reference's layout (CSGFoundry/*.npy + SSim/stree/standard) loads back to the same
    arrays and the same simulation."""
    from eic_opticks_gb300 import csgfoundry, geometry as G, gensteps as GS
    g, _ = __import__("eic_opticks_gb300.gdml", fromlist=["load"]).load(DOC)
    for arrays in (g.arrays(), G.crystal_array().arrays()):
        d = csgfoundry.save(arrays, str(tmp_path / ("x%d" % len(arrays["inst"]))))
        assert os.path.exists(os.path.join(d, "SSim", "stree", "standard", "bnd.npy"))
        back = csgfoundry.load(os.path.dirname(d))
        for k in ("node", "prim", "inst", "itra", "plan", "bnd", "optical", "icdf"):
            assert np.array_equal(np.asarray(back[k]).view(np.uint8), np.asarray(arrays[k]).view(np.uint8)), k
        assert np.array_equal(back["solid"].view(np.uint8), arrays["solid"].view(np.uint8))
        assert back["hd_factor"] == arrays["hd_factor"] and tuple(back["domain"]) == tuple(arrays["domain"])
    gs = GS.crystal_scint_gensteps(4, 100, seed=2)
    a, _ = oracle.simulate(oracle.SimConfig(arrays), gs)
    b, _ = oracle.simulate(oracle.SimConfig(back), gs)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_csgfoundry_loader_reads_reference_np_folder(oracle):
    """A folder written by the reference's own NP writer (sysrap/NP.hh, CSGFoundry::save_ layout with the
    SSim/stree/standard tables and their metadata; tests/golden/make_csgfoundry_golden.py) loads to exactly the
    arrays it was written from, and simulates the same photons."""
    from conftest import GOLDEN
    from eic_opticks_gb300 import csgfoundry
    z = load_golden("sim_csg_lists.npz")
    a = csgfoundry.load(os.path.join(GOLDEN, "csgfoundry_np", "csg_lists"))
    for k in ("node", "prim", "inst", "itra", "plan", "bnd", "optical", "icdf"):
        assert np.array_equal(np.asarray(a[k]).view(np.uint8), np.asarray(z[k]).view(np.uint8)), k
    assert np.array_equal(a["solid"].view(np.uint8), z["solid"].view(np.uint8))
    assert a["hd_factor"] == int(z["hd_factor"]) and tuple(a["domain"]) == tuple(float(x) for x in z["domain"])
    out, _ = oracle.simulate(oracle.SimConfig(a), z["gs"], event_index=int(z["event_index"]))
    assert np.array_equal(out.view(np.uint32), z["photon"].view(np.uint32))


@pytest.mark.skipif(not os.environ.get("GBO_REFERENCE_DIR"), reason="reference tree not available (GBO_REFERENCE_DIR)")
def test_reference_np_folder_fixture_is_current(tmp_path):
    """The committed folder is what the reference's NP writer writes today, file for file."""
    import importlib.util
    from conftest import GOLDEN
    spec = importlib.util.spec_from_file_location("mcg", os.path.join(GOLDEN, "make_csgfoundry_golden.py"))
    mcg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mcg)
    fresh = mcg.main(str(tmp_path), os.environ["GBO_REFERENCE_DIR"])
    committed = os.path.join(GOLDEN, "csgfoundry_np", "csg_lists")
    for base, _, files in os.walk(committed):
        for f in files:
            rel = os.path.relpath(os.path.join(base, f), committed)
            with open(os.path.join(committed, rel), "rb") as x, open(os.path.join(fresh, rel), "rb") as y:
                assert x.read() == y.read(), rel
