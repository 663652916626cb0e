"""A CSGFoundry folder written by the reference's own NP writer (tests/golden/csgfoundry_np/csg_lists/), for the
loader test in tests/test_gdml.py.  tests/cpp/np_foundry_writer.cc includes the reference's header-only
sysrap/NP.hh and writes the arrays of tests/golden/sim_csg_lists.npz (instances with transforms, a convex
polyhedron's planes, CSG list nodes, a sensor identity) in the CSGFoundry::save_ layout with the SSim/stree/standard
tables and their metadata.

    GBO_REFERENCE_DIR=<reference checkout> python tests/golden/make_csgfoundry_golden.py [outdir]
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def write_raw(z, d):
    """The fixture's arrays as the raw files and dims.txt np_foundry_writer reads."""
    arrays = {k: z[k] for k in ("node", "prim", "solid", "inst", "itra", "plan", "bnd", "optical", "icdf")}
    np.ascontiguousarray(arrays["solid"]).view(np.int32).tofile(os.path.join(d, "solid.bin"))
    for k in ("prim", "node", "inst", "itra", "plan"):
        np.ascontiguousarray(arrays[k], dtype=np.float32).tofile(os.path.join(d, k + ".bin"))
    np.zeros(0, np.float32).tofile(os.path.join(d, "tran.bin"))
    np.ascontiguousarray(arrays["bnd"], dtype=np.float64).tofile(os.path.join(d, "bnd.bin"))
    np.ascontiguousarray(arrays["optical"]).astype(np.int32).tofile(os.path.join(d, "optical.bin"))
    np.ascontiguousarray(arrays["icdf"], dtype=np.float64).tofile(os.path.join(d, "icdf.bin"))
    b = arrays["bnd"]
    dims = [len(arrays["solid"]), len(arrays["prim"]), len(arrays["node"]), len(arrays["inst"]),
            len(arrays["itra"]), 0, len(arrays["plan"]), b.shape[0], b.shape[3], arrays["icdf"].shape[0],
            arrays["icdf"].shape[1], int(z["hd_factor"])]
    lo, step = (float(x) for x in z["domain"])
    with open(os.path.join(d, "dims.txt"), "w") as f:
        f.write(" ".join(str(x) for x in dims) + " %r %r\n" % (lo, step))


def main(outdir, ref):
    z = np.load(os.path.join(HERE, "sim_csg_lists.npz"))
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "np_foundry_writer")
        subprocess.check_call(["g++", "-std=c++17", "-O1", "-w", "-I", os.path.join(ref, "sysrap"),
                               os.path.join(ROOT, "tests", "cpp", "np_foundry_writer.cc"), "-o", exe])
        raw = os.path.join(tmp, "raw")
        os.makedirs(raw)
        write_raw(z, raw)
        dest = os.path.join(outdir, "csg_lists")
        if os.path.isdir(dest):
            shutil.rmtree(dest)
        subprocess.check_call([exe, raw, dest])
    return dest


if __name__ == "__main__":
    ref = os.environ.get("GBO_REFERENCE_DIR")
    if not ref:
        sys.exit("set GBO_REFERENCE_DIR to a checkout of the reference")
    print(main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "csgfoundry_np"), ref))
