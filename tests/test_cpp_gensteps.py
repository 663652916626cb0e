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


def run_u4_check(tmp, n=400, env=None):
    exe = os.path.join(tmp, "gensteps_u4_check")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "gensteps_u4_check.cc"), "-o", exe])
    e = {k: v for k, v in os.environ.items() if not k.startswith("U4__CollectGenstep_")}
    e.update(env or {})
    out = subprocess.check_output([exe, tmp, str(n)], env=e, text=True)
    raw = np.fromfile(os.path.join(tmp, "inputs.bin"), dtype=np.uint8)
    v = raw[:n * 24 * 8].view(np.float64).reshape(n, 24)
    ints = raw[n * 24 * 8:].view(np.int32).reshape(n, 2)
    gs = np.fromfile(os.path.join(tmp, "gs.bin"), dtype=np.uint32).reshape(-1, 24)
    return v, ints, gs, out.split()


def reference_gensteps():
    import json
    with open(os.path.join(ROOT, "tests", "golden", "gensteps_ref.json")) as f:
        return json.load(f)


def test_genstep_codes_match_reference():
    """The genstep codes the producers and the engine use are the reference's OpticksGenstep_* values
    (sysrap/OpticksGenstep.h, read off the reference's header by oracle/ref_gensteps.cc)."""
    from eic_opticks_gb300 import layout as L
    en = reference_gensteps()["enums"]
    assert (L.GS_SCINTILLATION_R4695, L.GS_CERENKOV_MODIFIED, L.GS_TORCH, L.GS_SCINTILLATION, L.GS_CERENKOV) == \
        (en["DsG4Scintillation_r4695"], en["G4Cerenkov_modified"], en["TORCH"], en["SCINTILLATION"], en["CERENKOV"])


def test_gensteps_read_through_reference_structs(tmp_path):
    """Each field of a producer's genstep, read at the offset the reference's sscint / scerenkov struct gives it, holds
    the value u4/U4.cc:82-140 and :187-260 assign from the same step: positions, time, G4Step::GetDeltaPosition,
    G4Step::GetStepLength (the chord when the step length is not given), PDG code, charge, weight, the mean of the
    pre and post velocities, scnt and ScintillationTime; preVelocity, BetaInverse, Wmin / Wmax = h_Planck c_light /
    p / nm in CLHEP's units, maxCos, maxSin2, the two mean photon numbers and postVelocity."""
    ref = reference_gensteps()
    off, en = ref["offsets"], ref["enums"]
    n = 400
    v, ints, gs, _ = run_u4_check(str(tmp_path), n)
    f32 = gs.view(np.float32)

    def field(rows, name, k=0, kind="f"):
        w = off[name] // 4 + k
        return (f32 if kind == "f" else gs.view(np.int32) if kind == "i" else gs)[rows, w]

    sc, ck = np.arange(0, 2 * n, 2), np.arange(1, 2 * n, 2)
    pre, post = v[:, 0:3], v[:, 5:8]
    chord = np.sqrt(((post - pre) ** 2).sum(axis=1))
    step = np.where(v[:, 10] >= 0.0, v[:, 10], chord)
    for rows, st in ((sc, "sscint"), (ck, "scerenkov")):
        assert np.array_equal(field(rows, st + ".gentype", kind="u"),
                              np.full(n, en["DsG4Scintillation_r4695" if st == "sscint" else "G4Cerenkov_modified"]))
        assert np.array_equal(field(rows, st + ".trackid", kind="u"), v[:, 21].astype(np.uint32))
        assert np.array_equal(field(rows, st + ".matline", kind="u"), v[:, 23].astype(np.uint32))
        assert np.array_equal(field(rows, st + ".numphoton", kind="u"), ints[:, 0].astype(np.uint32))
        for k in range(3):
            assert np.array_equal(field(rows, st + ".pos", k), pre[:, k].astype(np.float32))
            assert np.array_equal(field(rows, st + ".DeltaPosition", k), (post[:, k] - pre[:, k]).astype(np.float32))
        assert np.array_equal(field(rows, st + ".time"), v[:, 3].astype(np.float32))
        assert np.array_equal(field(rows, st + ".step_length"), step.astype(np.float32))
        assert np.array_equal(field(rows, st + ".code", kind="i"), v[:, 22].astype(np.int32))
        assert np.array_equal(field(rows, st + ".charge"), v[:, 11].astype(np.float32))
        assert np.array_equal(field(rows, st + ".weight"), v[:, 12].astype(np.float32))
    assert np.array_equal(field(sc, "sscint.meanVelocity"), ((v[:, 4] + v[:, 9]) / 2.0).astype(np.float32))
    assert np.array_equal(field(sc, "sscint.scnt", kind="i"), ints[:, 1])
    assert np.array_equal(field(sc, "sscint.ScintillationTime"), v[:, 13].astype(np.float32))
    # CLHEP (Geant4's units: mm, ns, MeV), built as its headers build them
    MeV = 1.0; eV = 1.e-6 * MeV; joule = eV / 1.602176634e-19; s = 1.e+9; m = 1000.0; nm = 1.e-9 * m
    h_Planck = 6.62607015e-34 * joule * s
    c_light = 2.99792458e+8 * m / s
    wmin = h_Planck * c_light / (v[:, 16] * eV) / nm
    wmax = h_Planck * c_light / (v[:, 15] * eV) / nm
    assert np.array_equal(field(ck, "scerenkov.Wmin"), wmin.astype(np.float32))
    assert np.array_equal(field(ck, "scerenkov.Wmax"), wmax.astype(np.float32))
    # the same within a few binary32 ulp of the reference's own hc_eVnm (sysrap/smath.h) conversion
    assert np.allclose(field(ck, "scerenkov.Wmin"), 1239.8418754200 / v[:, 16], rtol=3e-7, atol=0)
    for name, col in (("preVelocity", 4), ("BetaInverse", 14), ("maxCos", 17), ("maxSin2", 18),
                      ("MeanNumberOfPhotons1", 19), ("MeanNumberOfPhotons2", 20), ("postVelocity", 9)):
        assert np.array_equal(field(ck, "scerenkov." + name), v[:, col].astype(np.float32)), name


def test_reference_demo_gensteps_from_the_producers(tmp_path):
    """The reference's demo gensteps (sscint::FillGenstep, scerenkov::FillGenstep) made from their values by the
    producers: every word but the genstep code (the demos use the generic SCINTILLATION / CERENKOV codes, U4.cc the
    r4695 / modified ones) and, for Cerenkov, Wmin / Wmax (the demo converts with binary32 smath::hc_eVnm, U4.cc with
    CLHEP's h_Planck c_light in binary64: within one binary32 ulp)."""
    ref = reference_gensteps()
    _, _, gs, _ = run_u4_check(str(tmp_path), ref["numphoton"])       # the demos carry that photon count
    scint = np.array([int(w, 16) for w in ref["scint_demo"]], dtype=np.uint32)
    cer = np.array([int(w, 16) for w in ref["cerenkov_demo"]], dtype=np.uint32)
    mine_s, mine_c = gs[-2], gs[-1]
    assert np.array_equal(mine_s[1:], scint[1:])
    wl = [ref["offsets"]["scerenkov.Wmin"] // 4, ref["offsets"]["scerenkov.Wmax"] // 4]
    keep = [i for i in range(1, 24) if i not in wl]
    assert np.array_equal(mine_c[keep], cer[keep])
    assert np.all(np.abs(mine_c[wl].astype(np.int64) - cer[wl].astype(np.int64)) <= 1)


def test_u4_collect_switches(tmp_path):
    """U4::CollectGenstep_*: the reference's DISABLE and ZEROPHO environment switches (u4/U4.cc:159-185, :278-311)."""
    _, _, _, out = run_u4_check(str(tmp_path), 2)
    assert out == ["2", "5:77", "18:88"]
    _, _, _, out = run_u4_check(str(tmp_path), 2, {"U4__CollectGenstep_DsG4Scintillation_r4695_DISABLE": "1",
                                                   "U4__CollectGenstep_G4Cerenkov_modified_ZEROPHO": "1"})
    assert out == ["1", "18:0"]


def test_reference_genstep_fixture_is_current(tmp_path):
    """The committed reference layouts and demo gensteps equal a fresh build of oracle/ref_gensteps.cc against the
    reference tree (skipped without GBO_REFERENCE_DIR)."""
    import json
    import pytest
    ref = os.environ.get("GBO_REFERENCE_DIR")
    if not ref or not os.path.isdir(os.path.join(ref, "sysrap")):
        pytest.skip("reference tree not available (GBO_REFERENCE_DIR)")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref-gensteps", "REFDIR=" + ref])
    out = subprocess.check_output([os.path.join(ROOT, "oracle", "_ref", "ref_gensteps"), "1000"], text=True)
    assert json.loads(out) == reference_gensteps()
