"""Child process of tests/test_gpu_parity.py: runs the engine's --fmad=false build (the library named by
GBO_ENGINE_LIBRARY) over the inputs of every reference-device fixture, in each kernel form, and writes one 64-bit
digest per photon (record and flag history) to the .npz path given as the argument.  A separate process because a
process loads one engine library."""
import importlib.util
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import __graft_entry__ as ge  # noqa: E402

ge.load_package()
from eic_opticks_gb300 import engine as E  # noqa: E402

_spec = importlib.util.spec_from_file_location("make_device_golden",
                                               os.path.join(ROOT, "tests", "golden", "make_device_golden.py"))
mdg = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(mdg)

# (kernel mode, Philox blocks by call): the four kernel modes, and three of them with Philox by call (a separate
# kernel form for geometries without CSG trees)
FORMS = ((2, 0), (1, 0), (0, 0), (3, 0), (2, 1), (1, 1), (3, 1))


def form_key(mode, rng_call):
    return "mode%d%s" % (mode, "_call" if rng_call else "")


def run(arrays, gs, inp, ev):
    out = {}
    for mode, rng_call in FORMS:
        eng = E.Engine(arrays, record_photon=1, record_seq=1, kernel_mode=mode, rng_call=rng_call)
        eng.simulate(ev, gs, inp)
        out[form_key(mode, rng_call)] = mdg.record_digest(eng.photons(), eng.seq()["seqhis"])
        eng.close()
    return out


def main(path):
    assert os.environ.get("GBO_ENGINE_LIBRARY", "").endswith("libgbopticks_nofma.so")
    res = {}
    for name in mdg.SIM_FIXTURES:
        z = np.load(os.path.join(ROOT, "tests", "golden", "sim_%s.npz" % name))
        inp = z["input_photon"] if len(z["input_photon"]) else None
        for form, d in run(mdg.golden_arrays(z), z["gs"], inp, int(z["event_index"])).items():
            res["%s_%s" % (name, form)] = d
    for name in mdg.CONFIGS:
        arrays, gs, inp, ev = mdg.config_inputs(name)
        for form, d in run(arrays, gs, inp, ev).items():
            res["%s_%s" % (name, form)] = d
    np.savez(path, **res)


if __name__ == "__main__":
    main(sys.argv[1])
