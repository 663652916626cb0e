"""CSGFoundry folder loader and writer: geometry exported by a reference install runs unchanged.

A reference install saves its translated geometry with ``CSGFoundry::save`` (CSG/CSGFoundry.cc:2769-2800):

    <dir>/CSGFoundry/solid.npy  (num_solid, 3, 4) int32   CSGSolid, 48 B (CSG/CSGSolid.h:37-52)
    <dir>/CSGFoundry/prim.npy   (num_prim, 4, 4)  float32 CSGPrim
    <dir>/CSGFoundry/node.npy   (num_node, 4, 4)  float32 CSGNode
    <dir>/CSGFoundry/plan.npy   (num_plan, 1, 4)  float32 planes (optional)
    <dir>/CSGFoundry/tran.npy, itra.npy (num_tran, 4, 4)  node transforms and their inverses (optional)
    <dir>/CSGFoundry/inst.npy   (num_inst, 4, 4)  float32 instance transforms, identities in the .w column

and the optical tables under ``SSim/stree/standard`` (SSim::RELDIR, stree::RELDIR, stree::STANDARD;
sysrap/sstandard.h:197-213): ``bnd.npy`` (num_bnd, 4, 2, 761, 4) float64 with the wavelength domain in its
metadata, ``optical.npy`` (num_bnd, 4, 4) int32 and ``icdf.npy`` (3, 4096) with its hd_factor.  NP keeps array
metadata in a ``<stem>_meta.txt`` sidecar of ``key:value`` lines.  ``load`` returns the engine's geometry arrays;
``save`` writes the same layout (for example from a GDML translation).
"""
import os

import numpy as np

from . import geometry as G
from . import layout as L

GEOM_FILES = ("solid", "prim", "node", "plan", "tran", "itra", "inst")
STANDARD = os.path.join("SSim", "stree", "standard")


def _meta(path):
    """NP metadata sidecar of an array file: {key: value-string}."""
    meta = {}
    side = path[:-4] + "_meta.txt"
    if os.path.exists(side):
        with open(side) as f:
            for line in f:
                if ":" in line:
                    k, v = line.split(":", 1)
                    meta[k.strip()] = v.strip()
    return meta


def _folder(path):
    cand = os.path.join(path, "CSGFoundry")
    return cand if os.path.isdir(cand) else path


def load(path):
    """Geometry arrays from a CSGFoundry folder (``path`` or ``path/CSGFoundry``)."""
    d = _folder(path)
    raw = {}
    for name in GEOM_FILES:
        f = os.path.join(d, name + ".npy")
        if os.path.exists(f):
            raw[name] = np.load(f, allow_pickle=False)
    for req in ("solid", "prim", "node", "inst"):
        if req not in raw:
            raise FileNotFoundError("CSGFoundry folder %s has no %s.npy" % (d, req))
    solid = np.ascontiguousarray(raw["solid"].astype(np.int32, copy=False)).reshape(-1, 12).view(L.SOLID).reshape(-1)
    out = dict(
        node=np.ascontiguousarray(raw["node"], dtype=np.float32).reshape(-1, 4, 4),
        prim=np.ascontiguousarray(raw["prim"], dtype=np.float32).reshape(-1, 4, 4),
        solid=solid,
        inst=np.ascontiguousarray(raw["inst"], dtype=np.float32).reshape(-1, 4, 4),
        itra=np.ascontiguousarray(raw.get("itra", np.zeros((0, 4, 4))), dtype=np.float32).reshape(-1, 4, 4),
        tran=np.ascontiguousarray(raw.get("tran", np.zeros((0, 4, 4))), dtype=np.float32).reshape(-1, 4, 4),
        plan=np.ascontiguousarray(raw.get("plan", np.zeros((0, 4))), dtype=np.float32).reshape(-1, 4),
    )
    std = os.path.join(d, STANDARD)
    bnd_path = os.path.join(std, "bnd.npy")
    if not os.path.exists(bnd_path):
        raise FileNotFoundError("no boundary table at %s" % bnd_path)
    bnd = np.load(bnd_path, allow_pickle=False)
    if bnd.ndim != 5 or bnd.shape[1:3] != (4, 2) or bnd.shape[4] != 4:
        raise ValueError("bnd.npy shape %s is not (num_bnd, 4, 2, nx, 4)" % (bnd.shape,))
    out["bnd"] = np.ascontiguousarray(bnd, dtype=np.float32)              # the reference narrows it too (QBnd)
    m = _meta(bnd_path)
    out["domain"] = (float(m.get("domain_low", G.DOMAIN_LOW)), float(m.get("domain_step", G.DOMAIN_STEP)))
    optical = np.load(os.path.join(std, "optical.npy"), allow_pickle=False)
    out["optical"] = np.ascontiguousarray(optical.astype(np.int64).astype(np.uint32)).reshape(-1, 4)
    icdf_path = os.path.join(std, "icdf.npy")
    if os.path.exists(icdf_path):
        out["icdf"] = np.ascontiguousarray(np.load(icdf_path, allow_pickle=False), dtype=np.float32).reshape(-1, 4096)
        out["hd_factor"] = int(float(_meta(icdf_path).get("hd_factor", 20)))
    else:
        out["icdf"] = G.default_icdf()
        out["hd_factor"] = 20
    return out


def save(arrays, path):
    """Write engine geometry arrays in the CSGFoundry + SSim/stree/standard layout under ``path/CSGFoundry``."""
    d = os.path.join(path, "CSGFoundry")
    std = os.path.join(d, STANDARD)
    os.makedirs(std, exist_ok=True)
    np.save(os.path.join(d, "solid.npy"), np.ascontiguousarray(arrays["solid"]).view(np.int32).reshape(-1, 3, 4))
    np.save(os.path.join(d, "prim.npy"), np.asarray(arrays["prim"], dtype=np.float32).reshape(-1, 4, 4))
    np.save(os.path.join(d, "node.npy"), np.asarray(arrays["node"], dtype=np.float32).reshape(-1, 4, 4))
    np.save(os.path.join(d, "inst.npy"), np.asarray(arrays["inst"], dtype=np.float32).reshape(-1, 4, 4))
    for name in ("tran", "itra"):
        a = np.asarray(arrays.get(name, np.zeros((0, 4, 4))), dtype=np.float32).reshape(-1, 4, 4)
        if len(a):
            np.save(os.path.join(d, name + ".npy"), a)
    plan = np.asarray(arrays.get("plan", np.zeros((0, 4))), dtype=np.float32).reshape(-1, 1, 4)
    if len(plan):
        np.save(os.path.join(d, "plan.npy"), plan)
    bnd_path = os.path.join(std, "bnd.npy")
    np.save(bnd_path, np.asarray(arrays["bnd"], dtype=np.float64))
    lo, step = arrays.get("domain", (G.DOMAIN_LOW, G.DOMAIN_STEP))
    nx = np.asarray(arrays["bnd"]).shape[3]
    with open(bnd_path[:-4] + "_meta.txt", "w") as f:
        f.write("domain_low:%g\ndomain_high:%g\ndomain_step:%g\n" % (lo, lo + step * (nx - 1), step))
    nb = np.asarray(arrays["bnd"]).shape[0]
    np.save(os.path.join(std, "optical.npy"), np.asarray(arrays["optical"]).astype(np.int32).reshape(nb, 4, 4))
    icdf_path = os.path.join(std, "icdf.npy")
    np.save(icdf_path, np.asarray(arrays["icdf"], dtype=np.float64))
    with open(icdf_path[:-4] + "_meta.txt", "w") as f:
        f.write("hd_factor:%d\n" % int(arrays.get("hd_factor", 20)))
    return d
