"""Golden fixtures for the reference's own GDML test geometries (tests/geom/*.gdml in the reference tree).

Run from the repository root in a checkout where the reference tree is available:

    make -C oracle ref && python tests/golden/make_gdml_golden.py [reference_root]

Each GDML file is translated by eic_opticks_gb300.gdml (no Geant4), and the photons of the reference's own tests
and configs are simulated by oracle/_ref/libref.so (the reference's qsim.h / csg_intersect_*.h headers compiled for
the host, curand's host Philox).  The translated arrays, the inputs and the reference outputs are written as
sim_gdml_<name>.npz in the layout of make_golden.py, so the GPU tests replay them without the reference tree.

Sources of the inputs:
* raindrop: the ten photons of tests/test_GPUPhotonFileSource.sh (pos (-10,-30,-90) mm, mom (0,0.287348,0.957826),
  pol (1,0,0), 3 x 420 nm, 2 x 450 nm, 5 x 500 nm) in tests/geom/opticks_raindrop.gdml; the reference test expects
  all ten to be hits with their wavelengths unchanged.  Its `-s 42` seeds Geant4's CLHEP engine; the Philox stream
  of the GPU simulation keeps the default seed 0.
* sipm8x8: config/8x8SiPM_crystal.json (torch disc r=0.5 mm at (-8.7,-8.7,4) mm along +z, 420 nm), 1000 photons,
  in tests/geom/8x8SiPM_w_CSI_optial_grease.gdml.
* sphere_leak: config/sphere_leak.json (torch disc r=0.1 mm at the origin along (0,0.3,1), 420 nm), 3000 photons
  (the config's 100000 cut for fixture size), in tests/geom/sphere_leak.gdml.
* basic_detector: 2000 isotropic 420 nm photons from the centre of tests/geom/basic_detector.gdml.
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import make_golden as MG  # noqa: E402
from eic_opticks_gb300 import gdml, gensteps as GS, layout as L  # noqa: E402

RAINDROP_WAVELENGTHS = [420.0] * 3 + [450.0] * 2 + [500.0] * 5


def raindrop_photons():
    p = np.zeros(10, dtype=L.PHOTON)
    p["pos"] = (-10.0, -30.0, -90.0)
    p["mom"] = (0.0, 0.287348, 0.957826)
    p["pol"] = (1.0, 0.0, 0.0)
    p["wavelength"] = RAINDROP_WAVELENGTHS
    return p


def torch(num, pos, mom, radius):
    return GS.torch_gensteps(1, num, torch_type=L.T_DISC, pos=pos, mom=mom, wavelength=420.0, radius=radius)


def main(ref_root):
    geom_dir = os.path.join(ref_root, "tests", "geom")
    g, _ = gdml.load(os.path.join(geom_dir, "opticks_raindrop.gdml"))
    ph = raindrop_photons()
    MG.sim_case("gdml_raindrop", g, GS.input_photon_genstep(len(ph)), ph)
    g, _ = gdml.load(os.path.join(geom_dir, "8x8SiPM_w_CSI_optial_grease.gdml"))
    MG.sim_case("gdml_sipm8x8", g, torch(1000, (-8.7, -8.7, 4.0), (0.0, 0.0, 1.0), 0.5))
    g, _ = gdml.load(os.path.join(geom_dir, "sphere_leak.gdml"))
    MG.sim_case("gdml_sphere_leak", g, torch(3000, (0.0, 0.0, 0.0), (0.0, 0.3, 1.0), 0.1))
    g, _ = gdml.load(os.path.join(geom_dir, "basic_detector.gdml"))
    iso = GS.isotropic_photons(2000, seed=21)
    MG.sim_case("gdml_basic_detector", g, GS.input_photon_genstep(len(iso)), iso)


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("GBO_REFERENCE_DIR")
    if not ref:
        sys.exit("usage: make_gdml_golden.py <reference checkout>  (or set GBO_REFERENCE_DIR)")
    main(ref)
