"""The G4CXOpticks-shaped C++ interface (include/G4CXOpticks_gb.hh) compiles against the C ABI and, on a GPU,
gives the same hits as the Python binding of the same entry points."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "g4cx_example.cc")


def compile_example(out_dir, src=SRC, name="g4cx_example", extra=()):
    import __graft_entry__ as ge
    ge.load_package()
    from eic_opticks_gb300 import build
    lib = build.build()
    exe = os.path.join(out_dir, name)
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"), src, "-o", exe,
                           lib, "-Wl,-rpath," + os.path.dirname(lib), *extra])
    return exe


def test_cpp_interface_compiles(tmp_path):
    exe = compile_example(str(tmp_path))
    assert os.path.exists(exe)


def test_event_api_example_compiles(tmp_path):
    """The engine-handle event API as a C caller binds it (tests/cpp/event_api_example.cc) compiles and links."""
    exe = compile_example(str(tmp_path), os.path.join(ROOT, "tests", "cpp", "event_api_example.cc"),
                          "event_api_example", ["-pthread"])
    assert os.path.exists(exe)


def write_inputs(d, arrays, gs, event_id):
    for k in ("node", "prim", "solid", "inst", "itra", "bnd", "optical", "icdf"):
        np.ascontiguousarray(arrays[k]).tofile(os.path.join(d, k + ".bin"))
    np.ascontiguousarray(gs).tofile(os.path.join(d, "gs.bin"))
    with open(os.path.join(d, "meta.txt"), "w") as f:
        f.write("%d %f %f %d %d\n" % (arrays["bnd"].shape[0], arrays["domain"][0], arrays["domain"][1],
                                      arrays["hd_factor"], event_id))


@pytest.mark.gpu
def test_cpp_interface_matches_python_binding(tmp_path):
    from eic_opticks_gb300 import engine as E, geometry as G, gensteps as GS
    arrays = G.crystal_array().arrays()
    gs = GS.crystal_scint_gensteps(20, 800, seed=4)
    exe = compile_example(str(tmp_path))
    write_inputs(str(tmp_path), arrays, gs, 3)
    out = subprocess.check_output([exe, str(tmp_path)]).decode().split()
    eng = E.Engine(arrays)
    n = eng.simulate(3, gs)
    hits = eng.hits()
    eng.close()
    assert int(out[1]) == n > 0
    assert int(out[3]) == hits["index"][0] and int(out[5]) == hits["index"][-1]


@pytest.mark.gpu
def test_event_api_example_matches_python_binding(tmp_path):
    """The C event-API example (four events from two threads) gives each event the hit count and first hit of
    gbo_simulate with the same event id."""
    from eic_opticks_gb300 import engine as E, geometry as G, gensteps as GS
    arrays = G.crystal_array().arrays()
    gs = GS.crystal_scint_gensteps(12, 600, seed=6)
    exe = compile_example(str(tmp_path), os.path.join(ROOT, "tests", "cpp", "event_api_example.cc"),
                          "event_api_example", ["-pthread"])
    write_inputs(str(tmp_path), arrays, gs, 20)
    lines = subprocess.check_output([exe, str(tmp_path)]).decode().strip().splitlines()
    assert len(lines) == 4
    eng = E.Engine(arrays)
    for line in lines:
        w = line.split()
        eid, n, first = int(w[1]), int(w[3]), int(w[6])
        assert eng.simulate(eid, gs) == n > 0
        assert eng.hits()["index"][0] == first
    eng.close()
