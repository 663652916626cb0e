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
                "gdml_raindrop", "gdml_sipm8x8", "gdml_sphere_leak", "gdml_basic_detector"]
