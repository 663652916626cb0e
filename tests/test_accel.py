"""Host-built acceleration structure (eic-opticks_gb300/csrc/gbo_accel.cpp) on the benchmark geometries and a
translated GDML geometry: TLAS coverage and box containment, containers under the root, overlap lists and clear
balls (tests/cpp/accel_check.cc).  No GPU: the builder is host code."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "eic-opticks_gb300", "csrc")


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    d = tmp_path_factory.mktemp("accel")
    exe = str(d / "accel_check")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                           "-I", CSRC, os.path.join(ROOT, "tests", "cpp", "accel_check.cc"),
                           os.path.join(CSRC, "gbo_accel.cpp"), "-o", exe])
    return exe


def geometries():
    from eic_opticks_gb300 import geometry as G
    yield "crystal_array", lambda: G.crystal_array().arrays()
    yield "water_cube", lambda: G.water_cube().arrays()
    yield "nested_boxes", lambda: G.nested_boxes(sensor=True).arrays()
    yield "large_sphere_2000", lambda: G.large_sphere(num_sensors=2000).arrays()


@pytest.mark.parametrize("name", [n for n, _ in geometries()])
def test_accel_invariants(checker, tmp_path, name):
    arrays = dict(geometries())[name]()
    for k in ("node", "prim", "solid", "inst"):
        np.ascontiguousarray(arrays[k]).tofile(str(tmp_path / ("%s.bin" % k)))
    out = subprocess.run([checker, str(tmp_path)], capture_output=True, text=True)
    print(name, out.stdout.strip())
    assert out.returncode == 0, out.stdout + out.stderr


def degenerate(kind):
    """Instance sets that defeat a surface-area split: thousands of coincident boxes, and a chain of box clusters at
    geometrically growing distances (each cluster 150 coincident boxes)."""
    from eic_opticks_gb300 import geometry as G
    g = G.Geometry("degenerate")
    m = G.Material("m")
    s = g.add_solid("b", [(G.box3(10, 10, 10), g.boundary(m, None, None, m))])
    if kind == "coincident":
        for _ in range(8000):
            g.add_instance(s, G.translate(1.0, 2.0, 3.0))
    else:
        for k in range(60):
            for _ in range(150):
                g.add_instance(s, G.translate(3.0 ** (k * 0.7), 0.0, 0.0))
    g.icdf = G.default_icdf()
    return g.arrays()


@pytest.mark.parametrize("kind", ["coincident", "chain"])
def test_accel_depth_bounded_on_degenerate_instances(checker, tmp_path, kind):
    """Degenerate instance sets either build within the traversal stack (the checker asserts the depth bound and
    every invariant above) or are refused with a message; a walk never drops a subtree."""
    arrays = degenerate(kind)
    for k in ("node", "prim", "solid", "inst"):
        np.ascontiguousarray(arrays[k]).tofile(str(tmp_path / ("%s.bin" % k)))
    out = subprocess.run([checker, str(tmp_path)], capture_output=True, text=True)
    print(kind, out.stdout.strip())
    assert out.returncode == 0 or "traversal stack" in out.stdout, out.stdout + out.stderr
    depth = int(out.stdout.split(" depth ")[1].split()[0])
    assert depth <= 64


@pytest.mark.parametrize("fixture", ["sim_gdml_sipm8x8.npz", "sim_gdml_basic_detector.npz", "sim_gdml_raindrop.npz"])
def test_accel_invariants_gdml(checker, tmp_path, fixture):
    """Geometries translated from the reference's GDML files (the arrays stored with their golden fixtures)."""
    from conftest import golden_arrays, load_golden
    arrays = golden_arrays(load_golden(fixture))
    for k in ("node", "prim", "solid", "inst"):
        np.ascontiguousarray(arrays[k]).tofile(str(tmp_path / ("%s.bin" % k)))
    out = subprocess.run([checker, str(tmp_path)], capture_output=True, text=True)
    print(fixture, out.stdout.strip())
    assert out.returncode == 0, out.stdout + out.stderr
