"""Host genstep producers (include/gbo_gensteps.hh): quad6 fields in the sscint / scerenkov layouts filled as
u4/U4.cc does, and the Cerenkov yield against a fine numerical integration of the same n(E)."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def run_example(tmp, env=None):
    exe = os.path.join(tmp, "gensteps_example")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "gensteps_example.cc"), "-o", exe])
    e = {k: v for k, v in os.environ.items() if not k.startswith("storch_FillGenstep_")}
    e.update(env or {})
    subprocess.check_call([exe, tmp], env=e)
    gs = np.fromfile(os.path.join(tmp, "gs.bin"), dtype=np.float32).reshape(-1, 6, 4)
    y = np.loadtxt(os.path.join(tmp, "yield.txt"))
    return gs, y


def water_table():
    wl = 200.0 + 500.0 * np.arange(36)[::-1] / 35.0
    return 1239.8418754200 / wl, 1.330 + 0.030 * (700.0 - wl) / 500.0


def fine_yield(beta, e, n, k=200000):
    ef = np.linspace(e[0], e[-1], k)
    nf = np.interp(ef, e, n)
    f = np.clip(1.0 - 1.0 / (beta * beta * nf * nf), 0.0, None)
    return 36.981 * np.trapezoid(f, ef)


def test_genstep_fields(tmp_path):
    from eic_opticks_gb300 import layout as L
    gs, y = run_example(str(tmp_path))
    u, i = gs.view(np.uint32), gs.view(np.int32)
    c = 299.792458
    # scintillation
    assert list(u[0, 0]) == [L.GS_SCINTILLATION_R4695, 7, 11, 4321]
    assert np.allclose(gs[0, 1], [10.0, -20.0, 30.0, 1.5])
    assert np.allclose(gs[0, 2, :3], [0.6, 0.8, 1.5], atol=1e-6) and abs(gs[0, 2, 3] - np.sqrt(0.36 + 0.64 + 2.25)) < 1e-6
    assert i[0, 3, 0] == 13 and gs[0, 3, 1] == -1.0 and gs[0, 3, 2] == 1.0
    assert abs(gs[0, 3, 3] - np.float32(0.94 * c)) < 1e-4 and i[0, 4, 0] == 1 and gs[0, 5, 0] == np.float32(12.5)
    # Cerenkov
    e, n = water_table()
    assert list(u[1, 0]) == [L.GS_CERENKOV_MODIFIED, 7, 7, 55]
    bi = 1.0 / 0.95
    assert abs(gs[1, 4, 0] - np.float32(bi)) < 1e-6
    assert abs(gs[1, 4, 1] - 200.0) < 1e-3 and abs(gs[1, 4, 2] - 700.0) < 1e-3          # Wmin, Wmax (nm)
    max_cos = bi / n.max()
    assert abs(gs[1, 4, 3] - np.float32(max_cos)) < 1e-6 and abs(gs[1, 5, 0] - np.float32(1 - max_cos ** 2)) < 1e-6
    step = np.sqrt(0.36 + 0.64 + 2.25)
    assert abs(gs[1, 5, 1] - fine_yield(0.95, e, n) * step) < 1e-3 * gs[1, 5, 1]
    assert abs(gs[1, 5, 2] - fine_yield(0.93, e, n) * step) < 1e-3 * gs[1, 5, 2]
    assert abs(gs[1, 3, 3] - np.float32(0.95 * c)) < 1e-4 and abs(gs[1, 5, 3] - np.float32(0.93 * c)) < 1e-4


def test_cerenkov_yield_against_fine_integration(tmp_path):
    _, y = run_example(str(tmp_path))
    e, n = water_table()
    for beta, got in y:
        want = fine_yield(beta, e, n)
        assert abs(got - want) <= 1e-4 * max(want, 1e-3) + 1e-6, (beta, got, want)
    assert y[0, 1] == 0.0                                   # below threshold (beta n < 1 everywhere)


def test_torch_genstep_defaults_and_environment(tmp_path):
    """MakeGenstep_Torch(TorchParamsFromEnv()) : storch::FillGenstep's fields, defaults and environment keys
    (sysrap/storch.h:104-146), the same record as the Python torch_gensteps with those parameters."""
    from eic_opticks_gb300 import gensteps as GS, layout as L
    gs, _ = run_example(str(tmp_path))
    want = GS.torch_gensteps(1, 1000)
    assert np.array_equal(gs[2].view(np.uint32), want[0].view(np.uint32))
    env = {"storch_FillGenstep_pos": "1,2,3", "storch_FillGenstep_mom": "0,3,4", "storch_FillGenstep_type": "sphere",
           "storch_FillGenstep_radius": "7.5", "storch_FillGenstep_wavelength": "500", "storch_FillGenstep_zenith": "0.1,0.2",
           "storch_FillGenstep_time": "2.5"}
    gs, _ = run_example(str(tmp_path), env)
    want = GS.torch_gensteps(1, 1000, torch_type=L.T_SPHERE, pos=(1, 2, 3), mom=(0, 3, 4), wavelength=500.0,
                             radius=7.5, zenith=(0.1, 0.2), time=2.5)
    assert np.array_equal(gs[2].view(np.uint32), want[0].view(np.uint32))
    gs, _ = run_example(str(tmp_path), {"storch_FillGenstep_type": "nonsense"})
    assert gs[2].view(np.uint32)[5, 3] == 0                        # undef: the reference asserts on it
