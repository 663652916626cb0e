import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as ge  # noqa: E402

ge.load_package()
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle():
    O = ge.load_oracle()
    O.build()
    return O


def load_golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def golden_arrays(z):
    keys = ("node", "prim", "solid", "inst", "itra", "plan", "bnd", "optical", "icdf")
    a = {k: z[k] for k in keys}
    a["hd_factor"] = int(z["hd_factor"])
    a["domain"] = tuple(float(x) for x in z["domain"])
    return a


SIM_FIXTURES = ["nested_boxes", "nested_boxes_sensor", "crystal_array", "water_cube", "torch", "large_sphere_small",
                "gdml_raindrop", "gdml_sipm8x8", "gdml_sphere_leak", "gdml_basic_detector", "csg_lists"]


# every shape of csg.npz: leaves, boolean trees, the convex polyhedron and the three list node kinds
CSG_SHAPES = ["sphere", "zsphere", "cylinder", "cone", "box3", "hyperboloid", "halfspace", "phicut", "ellipsoid",
              "difference", "intersection", "union3", "convexpolyhedron", "contiguous", "discontiguous", "overlap",
              "difference_list"]

INT_WORDS = [7, 12, 13, 14, 15]            # hitcount_iindex, orient_boundary_flag, identity, index, flagmask


def strict_fractions(a, b):
    """Fractions of photons whose positions agree within 1e-3 mm and times within 1e-3 ns (or one ulp of the value
    where that is larger)."""
    if len(a) == 0:
        return 1.0, 1.0
    pos_ok = np.all(np.abs(a["pos"] - b["pos"]) <= np.maximum(1e-3, np.spacing(np.abs(b["pos"]))), axis=1)
    t_ok = np.abs(a["time"] - b["time"]) <= np.maximum(1e-3, np.spacing(np.abs(b["time"])))
    return float(pos_ok.mean()), float(t_ok.mean())


def assert_photons_agree(a, b, pos_mm=1e-2, time_ns=1e-3, unit=1e-4):
    """Two kernels' photon records for the same photons: integer words identical, float words within bounds.

    Different kernels (one thread per photon, photon pool, no-allocation) are fused mul+add by ptxas differently
    under their own register budgets, so their binary32 results can differ in the last bits, which later steps
    can grow; the bounds are those of the reference parity (positions, times) and of a unit vector's rounding.
    Returns the largest differences seen."""
    wa, wb = a.view(np.uint32).reshape(-1, 16), b.view(np.uint32).reshape(-1, 16)
    assert np.array_equal(wa[:, INT_WORDS], wb[:, INT_WORDS])
    dpos = np.abs(a["pos"] - b["pos"]).max(initial=0.0)
    dt = np.abs(a["time"] - b["time"]).max(initial=0.0)
    dvec = max(np.abs(a["mom"] - b["mom"]).max(initial=0.0), np.abs(a["pol"] - b["pol"]).max(initial=0.0))
    dwl = np.abs(a["wavelength"] - b["wavelength"]).max(initial=0.0)
    assert dpos <= pos_mm and dt <= time_ns and dvec <= unit and dwl <= unit, (dpos, dt, dvec, dwl)
    return dpos, dt, dvec, dwl


def assert_forms_agree(a, b, fixture):
    """Two kernel forms' photons: integer words identical; float words within the kernel-form bounds, or, on a
    geometry whose mirrored paths amplify last-bit differences (ptxas fuses mul+add per kernel), positions and times
    within 1e-3 mm / 1e-3 ns for at least as many photons as the reference's own source built with and without
    contraction agree on (recorded in the reference-device fixture)."""
    try:
        assert_photons_agree(a, b)
    except AssertionError:
        d = load_golden("dev_" + fixture[len("sim_"):])
        pos, t = strict_fractions(a, b)
        assert pos >= min(0.999, float(d["self_pos"])) and t >= min(0.999, float(d["self_time"])), (pos, t)
