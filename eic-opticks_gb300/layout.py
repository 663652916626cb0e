"""numpy views of the reference's array layouts.

Each record type matches the byte layout the reference moves between host and device, so arrays built here
can be handed to the engine's C ABI and to a reference install alike:

* ``PHOTON``   sphoton, 64 B   (sysrap/sphoton.h:171-192)
* ``GENSTEP``  quad6, 96 B     (sysrap/squad.h; storch.h:43-69, scerenkov.h:29-58, sscint.h:34-62)
* ``NODE``     CSGNode, 64 B   (CSG/CSGNode.h:66-101)
* ``PRIM``     CSGPrim, 64 B   (CSG/CSGPrim.h:75-120)
* ``SOLID``    CSGSolid, 48 B  (CSG/CSGSolid.h:37-52)
* ``QAT4``     qat4, 64 B      (sysrap/sqat4.h)
"""
import numpy as np

PHOTON = np.dtype([
    ("pos", "<f4", 3), ("time", "<f4"),
    ("mom", "<f4", 3), ("hitcount_iindex", "<u4"),
    ("pol", "<f4", 3), ("wavelength", "<f4"),
    ("orient_boundary_flag", "<u4"), ("identity", "<u4"), ("index", "<u4"), ("flagmask", "<u4"),
])
assert PHOTON.itemsize == 64

SEQ = np.dtype([("seqhis", "<u8", 2), ("seqbnd", "<u8", 2)])
assert SEQ.itemsize == 32

SOLID = np.dtype([
    ("label", "S16"), ("numPrim", "<i4"), ("primOffset", "<i4"), ("type", "<i4"),
    ("intent", "S1"), ("pad", "S3"), ("center_extent", "<f4", 4),
])
assert SOLID.itemsize == 48

# photon flags : sysrap/OpticksPhoton.h:22-46
CERENKOV = 0x1 << 0
SCINTILLATION = 0x1 << 1
TORCH = 0x1 << 2
BULK_ABSORB = 0x1 << 3
BULK_REEMIT = 0x1 << 4
BULK_SCATTER = 0x1 << 5
SURFACE_DETECT = 0x1 << 6
SURFACE_ABSORB = 0x1 << 7
SURFACE_DREFLECT = 0x1 << 8
SURFACE_SREFLECT = 0x1 << 9
BOUNDARY_REFLECT = 0x1 << 10
BOUNDARY_TRANSMIT = 0x1 << 11
EFFICIENCY_COLLECT = 0x1 << 13
EFFICIENCY_CULL = 0x1 << 14
MISS = 0x1 << 15

FLAG_ABBREV = {
    CERENKOV: "CK", SCINTILLATION: "SI", TORCH: "TO", BULK_ABSORB: "AB", BULK_REEMIT: "RE",
    BULK_SCATTER: "SC", SURFACE_DETECT: "SD", SURFACE_ABSORB: "SA", SURFACE_DREFLECT: "DR",
    SURFACE_SREFLECT: "SR", BOUNDARY_REFLECT: "BR", BOUNDARY_TRANSMIT: "BT", MISS: "MI",
}

# genstep types : sysrap/OpticksGenstep.h:19-43
GS_SCINTILLATION_R4695 = 5
GS_TORCH = 6
GS_CERENKOV = 15
GS_SCINTILLATION = 16
GS_CERENKOV_MODIFIED = 18
GS_INPUT_PHOTON = 19

# torch types : sysrap/storchtype.h:10-18
T_DISC, T_LINE, T_POINT, T_CIRCLE, T_RECTANGLE, T_SPHERE_MARSAGLIA, T_SPHERE = 1, 2, 3, 4, 5, 6, 7

# CSG typecodes : sysrap/OpticksCSG.h
CSG_ZERO, CSG_UNION, CSG_INTERSECTION, CSG_DIFFERENCE = 0, 1, 2, 3
CSG_SPHERE, CSG_ZSPHERE, CSG_CYLINDER, CSG_CONE, CSG_BOX3 = 101, 103, 105, 108, 110
CSG_CONVEXPOLYHEDRON, CSG_HYPERBOLOID, CSG_PHICUT, CSG_HALFSPACE = 112, 117, 121, 125
CSG_CONTIGUOUS, CSG_DISCONTIGUOUS, CSG_OVERLAP = 11, 12, 13          # list nodes (csg_intersect_node.h)

# ems surface types : sysrap/smatsur.h:8-15
EMS_MATERIAL, EMS_NOSURFACE, EMS_SURFACE, EMS_ZPLUS_SENSOR_A = 0, 1, 2, 3


def hit_mask(spec="SD"):
    """OPTICKS_HIT_MASK style spec ("SD", "SD,EC") to a flag mask (sysrap/SEventConfig.cc:79)."""
    inv = {v: k for k, v in FLAG_ABBREV.items()}
    inv["EC"] = EFFICIENCY_COLLECT
    inv["EX"] = EFFICIENCY_CULL
    m = 0
    for tok in spec.split(","):
        tok = tok.strip()
        if tok:
            m |= inv[tok]
    return m


def flag_of(photons):
    return photons["orient_boundary_flag"] & 0xFFFF


def boundary_of(photons):
    return (photons["orient_boundary_flag"] >> 16) & 0x7FFF


def seqhis_str(seqhis_row):
    """Flag-history nibbles to the reference's "TO BT BT SA" style string."""
    out = []
    for w in seqhis_row:
        w = int(w)
        for s in range(16):
            nib = (w >> (4 * s)) & 0xF
            if nib == 0:
                return " ".join(out)
            out.append(FLAG_ABBREV.get(1 << (nib - 1), "?%d" % nib))
    return " ".join(out)
