"""Input-photon text files and the hit text format of the reference's photon-file application
(src/GPUPhotonFileSource.h): the C++ header (include/gbo_photon_file.hh) and the Python helpers
(eic_opticks_gb300.gensteps) read and write the same records."""
import os
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SAMPLE = """# x y z t mx my mz px py pz wl
-10 -30 -90 0 0 0.287348 0.957826 1 0 0 420

-10 -30 -90 0.5 0 0.287348 0.957826 1 0 0 450 trailing
not a photon line
1e-3 2.5 -3.25 1.25e2 0.6 0.8 0 0 0 1 399.5
1 2 3
1 2 3 4 0 0 1 1 0 0 1_0
1 2 3 4 0 0 1 1 0 0 nan
inf 2 3 4 0 0 1 1 0 0 400
1.5.5 3 4 0 0 1 1 0 0 400
0x1p3 2 3 4 0 0 1 1 0 0 400
1e 2 3 4 0 0 1 1 0 0 400
1 2 3 4 0 0 1 1 0 0 1e40
1 2 3 4 0 0 1 1 0 0 1e-45
1.000000059604644776257986737988403547205962240695953369140625 0 0 0 0 0 1 1 0 0 420
+5 -6 .5 5. 1E2 1e+2 0 1 0 0 420
--5 2 3 4 0 0 1 1 0 0 400
1 2 3 4 0 0 1 1 0 0 1_0 1 2 3
"""


def test_photon_file_roundtrip(tmp_path):
    from eic_opticks_gb300 import gensteps as GS, layout as L
    src = tmp_path / "photons.txt"
    src.write_text(SAMPLE)
    exe = str(tmp_path / "photon_file_example")
    subprocess.check_call(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "cpp", "photon_file_example.cc"), "-o", exe])
    subprocess.check_call([exe, str(src), str(tmp_path / "p.bin"), str(tmp_path / "hits_cpp.txt")])
    cpp = np.fromfile(str(tmp_path / "p.bin"), dtype=L.PHOTON)
    py = GS.load_photons_txt(str(src))
    # accepted: the three plain photons, "1_0" as the last value (reads 1), "1.5.5" (reads 1.5 then .5), the
    # underflowing 1e-45, the value that one rounding takes above 1.0, signs and exponent forms, the trailing tokens
    assert len(py) == len(cpp) == 9
    assert np.array_equal(py.view(np.uint32), cpp.view(np.uint32))
    assert py["wavelength"][1] == np.float32(450) and py["time"][2] == np.float32(125.0)
    assert py["wavelength"][3] == np.float32(1.0) and list(py["pos"][4]) == [1.5, 0.5, 3.0]
    assert py["wavelength"][5] == np.float32(1e-45) and py["wavelength"][5] > 0
    assert py["pos"][6].view(np.uint32)[0] == 0x3F800001           # 1 + 2^-23, not 1.0 (rounded once)
    assert list(py["pos"][7]) == [5.0, -6.0, 0.5] and py["time"][7] == 5.0
    GS.write_hits_txt(py, str(tmp_path / "hits_py.txt"))
    assert (tmp_path / "hits_py.txt").read_text() == (tmp_path / "hits_cpp.txt").read_text()
    assert (tmp_path / "hits_py.txt").read_text().splitlines()[0] == \
        "0 420  (-10, -30, -90)  (0, 0.287348, 0.957826)  (1, 0, 0)"


CONFIG = """{
  "torch": {"gentype": "TORCH", "trackid": 3, "matline": 5, "numphoton": 250,
            "pos": [1.0, -2.0, 4.5], "time": 0.25, "mom": [0.0, 3.0, 4.0], "weight": 0.0,
            "pol": [1.0, 0.0, 0.0], "wavelength": 440.0, "zenith": [0.0, 1.0], "azimuth": [0.0, 1.0],
            "radius": 2.5, "distance": 0.0, "mode": 255, "type": "circle"},
  "event": {"mode": "Minimal", "maxslot": 12345}
}"""


def test_torch_genstep_from_config(tmp_path):
    """A reference application config (gphox::Config::ReadConfig layout) gives the storch genstep field by field."""
    from eic_opticks_gb300 import gensteps as GS, layout as L
    p = tmp_path / "cfg.json"
    p.write_text(CONFIG)
    g, ev = GS.torch_genstep_from_config(str(p))
    u = g.view(np.uint32)
    assert g.shape == (1, 6, 4) and ev == {"mode": "Minimal", "maxslot": 12345}
    assert list(u[0, 0]) == [L.GS_TORCH, 3, 5, 250]
    assert list(g[0, 1]) == [1.0, -2.0, 4.5, 0.25]
    assert np.array_equal(g[0, 2, :3], np.array([0.0, 0.6, 0.8], dtype=np.float32)) and g[0, 2, 3] == 0.0
    assert list(g[0, 3]) == [1.0, 0.0, 0.0, 440.0]
    assert list(g[0, 4]) == [0.0, 1.0, 0.0, 1.0]
    assert g[0, 5, 0] == 2.5 and g[0, 5, 1] == 0.0 and u[0, 5, 2] == 255 and u[0, 5, 3] == L.T_CIRCLE
