"""Hit-merge fixtures (tests/golden/merge.npz) from the reference's own merge functors: oracle/_ref/ref_spm runs
sphoton::select_pred / key_functor / reduce_op (sysrap/sphoton.h:277-304) through thrust in the step order of
SPM::merge_partial_select (sysrap/SPM.cu:135-250).

    GBO_REFERENCE_DIR=<reference checkout> make -C oracle ref-spm && python tests/golden/make_merge_golden.py

Inputs, stored with the outputs: the hits of the reference-device crystal-array and 20,000-sensor samples
(dev_cfg2_crystal_array.npz, dev_cfg5_large_sphere.npz; at most 6,000 each) and a synthetic set with identities
above 16 bits, exact time ties and times on bucket edges; windows 0 (selection only), 1 and 10 ns, plus 0.37 ns for the synthetic set.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

ge.load_package()
from eic_opticks_gb300 import layout as L  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
REF_SPM = os.path.join(ROOT, "oracle", "_ref", "ref_spm")
SD = 1 << 6


def synthetic(n=20000, seed=17):
    rng = np.random.default_rng(seed)
    h = np.zeros(n, dtype=L.PHOTON)
    h["pos"] = rng.normal(size=(n, 3)).astype(np.float32)
    h["time"] = rng.uniform(0, 300.0, n).astype(np.float32)
    h["time"][rng.integers(0, n, n // 40)] = np.float32(3.0)                     # exact ties
    h["time"][rng.integers(0, n, n // 40)] = np.float32(10.0)                    # on bucket edges of 1 and 10 ns
    # 300 sensors, half the hits with the identity 65536 higher: the reference's key keeps 16 identity bits, so
    # those alias onto the same key and merge
    ids = rng.integers(1, 300, n).astype(np.uint32) + (rng.integers(0, 2, n).astype(np.uint32) << 16)
    h["identity"] = ids | (rng.integers(0, 2, n).astype(np.uint32) << 24)
    h["hitcount_iindex"] = (1 << 16) | rng.integers(0, 65536, n).astype(np.uint32)
    h["flagmask"] = SD | rng.integers(0, 1 << 12, n).astype(np.uint32)
    h["index"] = np.arange(n, dtype=np.uint32)
    return h


def ref_merge(hits, tw):
    with tempfile.TemporaryDirectory() as d:
        a, b = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        np.ascontiguousarray(hits).tofile(a)
        subprocess.check_call([REF_SPM, a, str(SD), repr(float(tw)), b], stdout=subprocess.DEVNULL)
        return np.fromfile(b, dtype=L.PHOTON)


def main():
    cases = {}
    for name, fixture in (("crystal", "dev_cfg2_crystal_array.npz"), ("large_sphere", "dev_cfg5_large_sphere.npz")):
        p = np.load(os.path.join(HERE, fixture))["photon"]
        cases[name] = p[(p["flagmask"] & SD) != 0][:6000]
    cases["synthetic"] = synthetic()
    out = {}
    for name, hits in cases.items():
        out[name + "_hits"] = hits
        windows = (0.0, 1.0, 10.0) + ((0.37,) if name == "synthetic" else ())
        for tw in windows:
            m = ref_merge(hits, tw)
            out["%s_tw%g" % (name, tw)] = m
            print("%s: %d hits, window %g ns -> %d" % (name, len(hits), tw, len(m)))
    path = os.path.join(HERE, "merge.npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    main()
