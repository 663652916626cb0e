"""Writes tests/golden/gensteps_ref.json: the reference's genstep struct layouts (field offsets of sysrap/sscint.h
and sysrap/scerenkov.h), its OpticksGenstep_* codes and its demo gensteps (sscint::FillGenstep,
scerenkov::FillGenstep), from oracle/ref_gensteps.cc compiled against the reference tree named by
GBO_REFERENCE_DIR (make -C oracle ref-gensteps)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))


def main():
    ref = os.environ.get("GBO_REFERENCE_DIR")
    if not ref or not os.path.isdir(os.path.join(ref, "sysrap")):
        sys.exit("set GBO_REFERENCE_DIR to the reference tree")
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref-gensteps", "REFDIR=" + ref])
    out = subprocess.check_output([os.path.join(ROOT, "oracle", "_ref", "ref_gensteps"), "1000"], text=True)
    d = json.loads(out)
    path = os.path.join(ROOT, "tests", "golden", "gensteps_ref.json")
    with open(path, "w") as f:
        json.dump(d, f, indent=1, sort_keys=True)
        f.write("\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
