"""Geometry and optical-property tables in the reference's CSGFoundry / boundary-texture layouts.

The reference receives its geometry from Geant4 through ``G4CXOpticks::SetGeometry`` (g4cx/G4CXOpticks.cc:315-346),
which translates the volume tree into CSGFoundry arrays (CSG/CSGFoundry.cc:2782-2788) and material/surface tables
(sysrap/sstandard.h:179-420).  Geant4 is outside the hot path, so this module builds the same arrays directly:

* ``node``   (num_node, 4, 4) f32   CSGNode   (CSG/CSGNode.h:66-101)
* ``prim``   (num_prim, 4, 4) f32   CSGPrim   (CSG/CSGPrim.h:75-120)
* ``solid``  (num_solid,)     SOLID CSGSolid  (CSG/CSGSolid.h:37-52)
* ``inst``   (num_inst, 4, 4) f32   forward instance transform, identity ints in the .w column (sysrap/sqat4.h:345-372)
* ``itra``   (num_tran, 4, 4) f32   inverse node transforms; ``tran`` holds the forward ones
* ``plan``   (num_plan, 4)    f32   convex polyhedron planes
* ``bnd``    (num_bnd, 4, 2, 761, 4) f32 boundary texture payload: per boundary (omat, osur, isur, imat), two
  float4 groups, on the 60-820 nm 1 nm domain (sysrap/sdomain.h:23-40, qudarap/qbnd.h:103-125)
* ``optical`` (num_bnd*4, 4) u32    (sysrap/sstandard.h:262-420)
* ``icdf``   (3, 4096)        f32   scintillation inverse CDF with hd_factor 20 (u4/U4Scint.h:426-484)

Builders for the five benchmark geometries follow at the end of the module.
"""
import math
import numpy as np

from . import layout as L

DOMAIN_LOW, DOMAIN_HIGH, DOMAIN_STEP = 60.0, 820.0, 1.0
DOMAIN = np.linspace(DOMAIN_LOW, DOMAIN_HIGH, 761)
C_LIGHT = 299.792458          # mm/ns, GROUPVEL default (sysrap/sproplist.h:37)
HC_EVNM = 1239.8418754200     # h c in eV nm (sysrap/smath.h:13)


# ---------------------------------------------------------------------------------------------------------------
# materials and surfaces

def _on_domain(v):
    if callable(v):
        return np.asarray(v(DOMAIN), dtype=np.float64)
    arr = np.asarray(v, dtype=np.float64)
    if arr.ndim == 0:
        return np.full(DOMAIN.shape, float(arr))
    if arr.ndim == 1 and arr.shape == DOMAIN.shape:      # already sampled on the domain
        return arr
    if arr.ndim == 2:                      # (n, 2) table of (wavelength_nm, value): clamp outside its range
        order = np.argsort(arr[:, 0])
        return np.interp(DOMAIN, arr[order, 0], arr[order, 1])
    raise ValueError("property must be scalar, callable or (n,2) table")


class Material:
    """Material property set on the 761-bin domain; defaults follow sysrap/sproplist.h:31-40."""

    def __init__(self, name, rindex=1.0, abslength=1e12, rayleigh=1e12, reemprob=0.0, groupvel=None):
        self.name = name
        self.rindex = _on_domain(rindex)
        self.abslength = _on_domain(abslength)
        self.rayleigh = _on_domain(rayleigh)
        self.reemprob = _on_domain(reemprob)
        if groupvel is None:
            # c / n_g with n_g = n - lambda dn/dlambda (the dispersion relation Geant4 applies when GROUPVEL is
            # derived from RINDEX); flat n gives c/n.
            n = self.rindex
            dn = np.gradient(n, DOMAIN)
            ng = n - DOMAIN * dn
            self.groupvel = C_LIGHT / ng
        else:
            self.groupvel = _on_domain(groupvel)

    def payload(self):
        p = np.zeros((2, 761, 4), dtype=np.float32)
        p[0, :, 0] = self.rindex
        p[0, :, 1] = self.abslength
        p[0, :, 2] = self.rayleigh
        p[0, :, 3] = self.reemprob
        p[1, :, 0] = self.groupvel
        return p


class Surface:
    """Surface payload (detect, absorb, reflect_specular, reflect_diffuse), summing to one.

    Follows u4/U4SurfaceArray.h:159-240: a sensor gives detect=eff, absorb=1-eff; a polished non-sensor gives
    specular=R, absorb=1-R; any other finish gives diffuse=R, absorb=1-R.
    """

    def __init__(self, name, detect=0.0, absorb=0.0, specular=0.0, diffuse=0.0, ems=L.EMS_SURFACE, finish=0,
                 value_percent=0):
        self.name = name
        self.detect, self.absorb, self.specular, self.diffuse = (_on_domain(x) for x in (detect, absorb, specular, diffuse))
        self.ems = ems
        self.finish = finish
        self.value_percent = value_percent

    @classmethod
    def sensor(cls, name, efficiency):
        return cls(name, detect=efficiency, absorb=1.0 - efficiency)

    @classmethod
    def polished(cls, name, reflectivity):
        return cls(name, absorb=1.0 - reflectivity, specular=reflectivity, finish=0)

    @classmethod
    def ground(cls, name, reflectivity):
        return cls(name, absorb=1.0 - reflectivity, diffuse=reflectivity, finish=3)

    @classmethod
    def absorber(cls, name):
        return cls(name, absorb=1.0)

    def payload(self):
        p = np.zeros((2, 761, 4), dtype=np.float32)
        p[0, :, 0] = self.detect
        p[0, :, 1] = self.absorb
        p[0, :, 2] = self.specular
        p[0, :, 3] = self.diffuse
        return p


# ---------------------------------------------------------------------------------------------------------------
# transforms

def translate(x, y, z):
    m = np.eye(4)
    m[3, :3] = (x, y, z)          # row-vector convention: translation in the last row (sysrap/sqat4.h:45-52)
    return m


def scale(sx, sy, sz):
    return np.diag([sx, sy, sz, 1.0])


def rotate_z_to(direction):
    """Rotation (row-vector convention) taking local +z onto ``direction``."""
    d = np.asarray(direction, dtype=np.float64)
    d = d / np.linalg.norm(d)
    a = np.array([0.0, 0.0, 1.0]) if abs(d[2]) < 0.9 else np.array([1.0, 0.0, 0.0])
    x = np.cross(a, d)
    x /= np.linalg.norm(x)
    y = np.cross(d, x)
    m = np.eye(4)
    m[0, :3] = x
    m[1, :3] = y
    m[2, :3] = d
    return m


# ---------------------------------------------------------------------------------------------------------------
# CSG nodes

def _node(typecode, q0=(0, 0, 0, 0), q1xy=(0, 0), bbox=None, complement=False):
    return dict(typecode=typecode, q0=tuple(float(v) for v in q0), q1xy=tuple(float(v) for v in q1xy),
                bbox=bbox, complement=complement, transform=None)


def box3(fx, fy, fz):
    return _node(L.CSG_BOX3, (fx, fy, fz, 0.0), bbox=(-fx / 2, -fy / 2, -fz / 2, fx / 2, fy / 2, fz / 2))


def sphere(r, center=(0.0, 0.0, 0.0)):
    cx, cy, cz = center
    return _node(L.CSG_SPHERE, (cx, cy, cz, r), bbox=(cx - r, cy - r, cz - r, cx + r, cy + r, cz + r))


def zsphere(r, z1, z2, center=(0.0, 0.0, 0.0)):
    cx, cy, cz = center
    return _node(L.CSG_ZSPHERE, (cx, cy, cz, r), (z1, z2), bbox=(cx - r, cy - r, cz + z1, cx + r, cy + r, cz + z2))


def cylinder(r, z1, z2):
    return _node(L.CSG_CYLINDER, (0.0, 0.0, 0.0, r), (z1, z2), bbox=(-r, -r, z1, r, r, z2))


def cone(r1, z1, r2, z2):
    rm = max(r1, r2)
    return _node(L.CSG_CONE, (r1, z1, r2, z2), bbox=(-rm, -rm, z1, rm, rm, z2))


def convexpolyhedron(planes, bbox):
    """Convex polyhedron leaf: planes (n, 4) as (outward normal, distance from the origin); the planes go into the
    geometry's plan array when the solid is added (CSG/csg_intersect_leaf_convexpolyhedron.h:40-106)."""
    nd = _node(L.CSG_CONVEXPOLYHEDRON, bbox=tuple(float(v) for v in bbox))
    nd["planes"] = np.asarray(planes, dtype=np.float64).reshape(-1, 4)
    return nd


def with_transform(node, m):
    node = dict(node)
    node["transform"] = np.asarray(m, dtype=np.float64) if node.get("transform") is None else node["transform"] @ m
    return node


def operation(op, left, right):
    return dict(typecode=op, left=left, right=right)


def csg_list(typecode, leaves):
    """A CSG list node (CSG_CONTIGUOUS multi-union of overlapping leaves, CSG_DISCONTIGUOUS union of disjoint
    leaves, CSG_OVERLAP multi-intersection; CSG/csg_intersect_node.h): a prim of its own or a leaf of a boolean
    tree.  Its leaves are stored after the prim's tree nodes and addressed by subNum / subOffset (CSGNode.h:210)."""
    assert typecode in (L.CSG_CONTIGUOUS, L.CSG_DISCONTIGUOUS, L.CSG_OVERLAP) and leaves
    assert all("left" not in x and "subs" not in x for x in leaves)
    return dict(typecode=typecode, subs=list(leaves))


def _transform_bbox(bb, m):
    if m is None:
        return bb
    corners = np.array([[x, y, z, 1.0] for x in (bb[0], bb[3]) for y in (bb[1], bb[4]) for z in (bb[2], bb[5])])
    t = corners @ m
    return (*t[:, :3].min(axis=0), *t[:, :3].max(axis=0))


def _tree_nodes(tree):
    """Complete binary tree in level order, CSG_ZERO fillers (CSG/csg_postorder.h layout)."""
    def height(t):
        return 0 if "left" not in t else 1 + max(height(t["left"]), height(t["right"]))
    h = height(tree)
    n = (1 << (h + 1)) - 1
    out = [None] * n

    def place(t, i):
        out[i] = t
        if "left" in t:
            place(t["left"], 2 * i + 1)
            place(t["right"], 2 * i + 2)
    place(tree, 0)
    return out


class Geometry:
    """Accumulates solids, prims, nodes, instances and boundaries into CSGFoundry-layout arrays."""

    def __init__(self, name="geometry"):
        self.name = name
        self.materials, self.surfaces, self.boundaries = [], [], []
        self._nodes, self._prims, self._solids, self._tran, self._inst = [], [], [], [], []
        self.plan = np.zeros((0, 4), dtype=np.float32)
        self.icdf = None
        self.hd_factor = 20

    # -- optical properties ----------------------------------------------------------------------------------
    def material(self, m):
        for i, x in enumerate(self.materials):
            if x.name == m.name:
                return i
        self.materials.append(m)
        return len(self.materials) - 1

    def surface(self, s):
        if s is None:
            return -1
        for i, x in enumerate(self.surfaces):
            if x.name == s.name:
                return i
        self.surfaces.append(s)
        return len(self.surfaces) - 1

    def boundary(self, omat, osur, isur, imat):
        key = (self.material(omat), self.surface(osur), self.surface(isur), self.material(imat))
        if key in self.boundaries:
            return self.boundaries.index(key)
        self.boundaries.append(key)
        return len(self.boundaries) - 1

    def material_line(self, bnd, which=L.EMS_MATERIAL):
        """Texture line of the inner material of boundary ``bnd`` (genstep matline after SEvt::addGenstep)."""
        return 4 * bnd + 3

    # -- shapes --------------------------------------------------------------------------------------------
    def add_solid(self, label, prims):
        """prims: list of (tree_or_leaf, boundary).  Returns solid index."""
        prim_offset = len(self._prims)
        lo = np.full(3, np.inf)
        hi = np.full(3, -np.inf)
        for tree, bnd in prims:
            nodes = _tree_nodes(tree) if "left" in tree else [tree]
            node_offset = len(self._nodes)
            bbs = []
            subs = []                      # leaves of list nodes, stored after the tree nodes
            for nd in nodes:
                rec = np.zeros((4, 4), dtype=np.float32)
                ints = rec.view(np.uint32)
                if nd is None:
                    ints[3, 2] = L.CSG_ZERO
                    ints[1, 2] = bnd
                elif "left" in nd:
                    ints[3, 2] = nd["typecode"]
                    ints[1, 2] = bnd
                elif "subs" in nd:
                    ints[3, 2] = nd["typecode"]
                    ints[1, 2] = bnd
                    ints[0, 0] = len(nd["subs"])                 # subNum
                    ints[0, 1] = len(nodes) + len(subs)          # subOffset from the prim's root
                    sb = np.array([_transform_bbox(x["bbox"], x.get("transform")) for x in nd["subs"]])
                    bb = (*sb[:, 0:3].min(axis=0), *sb[:, 3:6].max(axis=0))
                    if nd["typecode"] == L.CSG_OVERLAP:         # an intersection lies inside every leaf
                        bb = (*sb[:, 0:3].max(axis=0), *sb[:, 3:6].min(axis=0))
                    rec[2, :] = bb[0:4]
                    rec[3, 0:2] = bb[4:6]
                    bbs.append(bb)
                    subs.extend(nd["subs"])
                else:
                    rec, bb = self._leaf_record(nd, bnd)
                    if bb is not None:
                        bbs.append(bb)
                    ints = rec.view(np.uint32)
                ints[1, 3] = len(self._nodes) - node_offset
                self._nodes.append(rec)
            if len(nodes) > 1:
                self._nodes[node_offset].view(np.uint32)[0, 0] = len(nodes)   # subNum on the root
                self._nodes[node_offset].view(np.uint32)[0, 1] = 0
            for leaf in subs:
                rec, _ = self._leaf_record(leaf, bnd)
                rec.view(np.uint32)[1, 3] = len(self._nodes) - node_offset
                self._nodes.append(rec)
            bb = np.array(bbs)
            plo, phi = bb[:, 0:3].min(axis=0), bb[:, 3:6].max(axis=0)
            lo, hi = np.minimum(lo, plo), np.maximum(hi, phi)
            prec = np.zeros((4, 4), dtype=np.float32)
            pi = prec.view(np.int32)
            pi[0, 0] = len(nodes) + len(subs)
            pi[0, 1] = node_offset
            pu = prec.view(np.uint32)
            pu[1, 2] = len(self._solids)
            pu[1, 3] = len(self._prims) - prim_offset
            prec[2, 0:3] = plo
            prec[2, 3] = phi[0]
            prec[3, 0:2] = phi[1:3]
            pu[3, 3] = len(self._prims)                 # globalPrimIdx
            self._prims.append(prec)
        center = (lo + hi) / 2
        extent = float(np.max(hi - lo) / 2)
        self._solids.append((label, len(prims), prim_offset, (*center, extent)))
        return len(self._solids) - 1

    def _leaf_record(self, nd, bnd):
        """The CSGNode record of a leaf and its bounding box (None for a complemented leaf)."""
        rec = np.zeros((4, 4), dtype=np.float32)
        ints = rec.view(np.uint32)
        rec[0, :] = nd["q0"]
        rec[1, 0:2] = nd["q1xy"]
        if nd.get("planes") is not None:             # planeIdx, planeNum (CSGNode::setPlaneIdx/Num)
            ints[0, 0] = len(self.plan)
            ints[0, 1] = len(nd["planes"])
            self.plan = np.concatenate([self.plan, nd["planes"].astype(np.float32)])
        ints[1, 2] = bnd
        ints[3, 2] = nd["typecode"]
        tidx = 0
        if nd.get("transform") is not None:
            self._tran.append(nd["transform"])
            tidx = len(self._tran)          # 1-based
        ints[3, 3] = (tidx & 0x7FFFFFFF) | (0x80000000 if nd.get("complement") else 0)
        bb = _transform_bbox(nd["bbox"], nd.get("transform"))
        rec[2, :] = bb[0:4]
        rec[3, 0:2] = bb[4:6]
        return rec, (None if nd.get("complement") else bb)

    def add_instance(self, solid, transform=None, sensor_identifier=-1, sensor_index=-1):
        m = np.eye(4) if transform is None else np.asarray(transform, dtype=np.float64)
        q = m.astype(np.float32).copy()
        qi = q.view(np.int32)
        qi[0, 3] = len(self._inst)
        qi[1, 3] = solid
        qi[2, 3] = sensor_identifier + 1          # 0 means not a sensor (sysrap/sqat4.h:367-372)
        qi[3, 3] = sensor_index
        self._inst.append(q)
        return len(self._inst) - 1

    # -- finalize -------------------------------------------------------------------------------------------
    def arrays(self):
        node = np.array(self._nodes, dtype=np.float32).reshape(-1, 4, 4)
        prim = np.array(self._prims, dtype=np.float32).reshape(-1, 4, 4)
        solid = np.zeros(len(self._solids), dtype=L.SOLID)
        for i, (label, n, off, ce) in enumerate(self._solids):
            solid[i]["label"] = label.encode()[:16]
            solid[i]["numPrim"] = n
            solid[i]["primOffset"] = off
            solid[i]["center_extent"] = ce
        inst = np.array(self._inst, dtype=np.float32).reshape(-1, 4, 4)
        tran = np.array([t for t in self._tran], dtype=np.float64).reshape(-1, 4, 4)
        itra = np.array([np.linalg.inv(t) for t in self._tran], dtype=np.float64).reshape(-1, 4, 4)
        for arr in (tran, itra):
            arr[:, :, 3] = (0, 0, 0, 1)
        nb = len(self.boundaries)
        bnd = np.zeros((nb, 4, 2, 761, 4), dtype=np.float32)
        optical = np.zeros((nb * 4, 4), dtype=np.uint32)
        for b, (om, os_, is_, im) in enumerate(self.boundaries):
            for j, (kind, idx) in enumerate((("m", om), ("s", os_), ("s", is_), ("m", im))):
                line = 4 * b + j
                if kind == "m":
                    bnd[b, j] = self.materials[idx].payload()
                    optical[line] = (idx + 1, 0, 0, 0)
                elif idx >= 0:
                    s = self.surfaces[idx]
                    bnd[b, j] = s.payload()
                    optical[line] = (idx + 1, s.ems, s.finish, s.value_percent)
                else:
                    optical[line] = (0, L.EMS_NOSURFACE, 0, 0)
        icdf = self.icdf if self.icdf is not None else default_icdf()
        return dict(node=node, prim=prim, solid=solid, inst=inst, itra=itra.astype(np.float32),
                    tran=tran.astype(np.float32), plan=self.plan.astype(np.float32), bnd=bnd, optical=optical,
                    icdf=icdf.astype(np.float32), hd_factor=self.hd_factor, domain=(DOMAIN_LOW, DOMAIN_STEP))


def invert_instances(inst):
    """Inverse instance transforms (object <- world), identity columns cleared."""
    m = inst.astype(np.float64).copy()
    m[:, :, 3] = (0, 0, 0, 1)
    inv = np.linalg.inv(m)
    inv[:, :, 3] = (0, 0, 0, 1)
    return inv.astype(np.float32)


# ---------------------------------------------------------------------------------------------------------------
# scintillation inverse CDF (u4/U4Scint.h:426-484 with hd_factor 20)

def scint_icdf(emission, num_bins=4096, hd_factor=20, num_table=256, lo=200.0, hi=800.0):
    """Inverse CDF of an emission spectrum given as a function of wavelength (nm).

    The spectrum is tabulated on ``num_table`` wavelength bins, integrated over photon energy (as Geant4 builds
    its ScintillationIntegral) and inverted by linear interpolation; the three rows hold the full range and the
    two hd_factor-times finer tails, sampled at u = j/num_bins as the reference does.
    """
    wl = np.linspace(lo, hi, num_table)
    e = HC_EVNM / wl[::-1]                           # increasing energy
    return scint_icdf_table(e, emission(wl[::-1]), num_bins, hd_factor)


def scint_icdf_table(energy_ev, intensity, num_bins=4096, hd_factor=20):
    """Inverse CDF of an emission spectrum tabulated at increasing photon energies (eV): the trapezoid running
    integral on the table's own points (u4/U4Scint.h:218-256, Geant4's ScintillationIntegral) inverted by linear
    interpolation, in the three-row hd_factor layout."""
    e = np.asarray(energy_ev, dtype=np.float64)
    f = np.asarray(intensity, dtype=np.float64)
    integ = np.concatenate([[0.0], np.cumsum(0.5 * (f[1:] + f[:-1]) * np.diff(e))])
    mx = integ[-1]
    j = np.arange(num_bins, dtype=np.float64)
    edge = 1.0 / hd_factor
    u_all = j / num_bins
    u_lhs = j / (hd_factor * num_bins)
    u_rhs = 1.0 - edge + j / (hd_factor * num_bins)
    out = np.zeros((3, num_bins), dtype=np.float64)
    for r, u in enumerate((u_all, u_lhs, u_rhs)):
        energy = np.interp(u * mx, integ, e)
        out[r] = HC_EVNM / energy
    return out.astype(np.float32)


def default_icdf():
    return scint_icdf(lambda w: np.exp(-0.5 * ((w - 430.0) / 30.0) ** 2))


# ---------------------------------------------------------------------------------------------------------------
# benchmark geometries

def nested_boxes(sensor=False):
    """Vacuum 240 / lead 220 / air 200 / water 100 mm cubes centred on the origin.

    ``sensor=True`` adds a water->air border surface of efficiency 1 (the raindrop fixture's medium_container_bs)
    so that hit compaction has work.
    """
    g = Geometry("nested_boxes" + ("_sensor" if sensor else ""))
    vac = Material("Vacuum", rindex=1.0)
    lead = Material("Lead", rindex=1.0, abslength=1e-6)
    air = Material("Air", rindex=1.0003, abslength=1e6)
    water = Material("Water", rindex=1.333, abslength=2e4, rayleigh=5e4)
    b_world = g.boundary(vac, None, None, vac)
    b_lead = g.boundary(vac, None, None, lead)
    b_air = g.boundary(lead, None, None, air)
    b_water = g.boundary(air, None, Surface.sensor("WaterAirSensor", 1.0) if sensor else None, water)
    s0 = g.add_solid("nested", [(box3(240, 240, 240), b_world), (box3(220, 220, 220), b_lead),
                                (box3(200, 200, 200), b_air), (box3(100, 100, 100), b_water)])
    g.add_instance(s0)
    g.icdf = default_icdf()
    return g


CRYSTAL_PITCH = 20.5


def crystal_array(n=8):
    """8x8 CsI crystals 20x20x200 mm with 0.5 mm air gaps, polished R=0.98 wrapping, 6x6 mm SiPM on each back face.

    Each crystal is one instance of a two-prim solid: the CsI box (crystal->air border surface: polished,
    specular 0.98 / absorb 0.02) and, flush with the +z back face inside it, a 6x6x0.5 mm SiPM whose
    CsI->SiPM surface detects with efficiency 0.40 and absorbs the rest.  The instance carries the crystal
    number as its sensor identifier.  The world is air.
    """
    g = Geometry("crystal_array")
    air = Material("Air", rindex=1.0003, abslength=1e6)
    csi = Material("CsI", rindex=1.79, abslength=1000.0)
    si = Material("Silicon", rindex=3.5, abslength=1e-3)
    wrap = Surface.polished("CsIWrap", 0.98)
    sipm = Surface.sensor("SiPMSensor", 0.40)
    b_world = g.boundary(air, None, None, air)
    b_crystal = g.boundary(air, None, wrap, csi)
    b_sipm = g.boundary(csi, sipm, None, si)
    half = n * CRYSTAL_PITCH / 2 + 20.0
    s0 = g.add_solid("world", [(box3(2 * half, 2 * half, 260.0), b_world)])
    s1 = g.add_solid("crystal", [(box3(20.0, 20.0, 200.0), b_crystal),
                                 (with_transform(box3(6.0, 6.0, 0.5), translate(0, 0, 100.0 - 0.25)), b_sipm)])
    g.add_instance(s0)
    for i in range(n):
        for j in range(n):
            x = (i - (n - 1) / 2) * CRYSTAL_PITCH
            y = (j - (n - 1) / 2) * CRYSTAL_PITCH
            g.add_instance(s1, translate(x, y, 0.0), sensor_identifier=i * n + j, sensor_index=i * n + j)
    g.icdf = scint_icdf(lambda w: np.exp(-0.5 * ((w - 550.0) / 50.0) ** 2))
    return g


def water_refractive_index_table():
    """36-point table 200-700 nm, linear from 1.360 at 200 nm to 1.330 at 700 nm."""
    wl = np.linspace(200.0, 700.0, 36)
    n = 1.360 + (wl - 200.0) * (1.330 - 1.360) / 500.0
    return np.stack([wl, n], axis=1)


def water_cube(detectors_per_face=4):
    """1 m water cube in a 1.2 m air cube lined with 64 r=40 mm disc detectors of efficiency 0.3.

    The reference GPU build has no disc leaf (CSG_DISC only under CSG_EXTRA), so each detector is a 0.1 mm thick
    cylinder.  Detectors sit on the four side walls of the air cube, 16 per wall, facing inwards; the inner face of
    the air cube carries an absorbing surface so that escaping photons end there.
    """
    g = Geometry("water_cube")
    air = Material("Air", rindex=1.0003, abslength=1e6)
    water = Material("Water", rindex=water_refractive_index_table(), abslength=1e4, rayleigh=3e4)
    det = Material("Detector", rindex=1.5, abslength=1e-3)
    black = Surface.absorber("WallAbsorber")
    sens = Surface.sensor("DiscSensor", 0.3)
    b_world = g.boundary(air, None, black, air)
    b_water = g.boundary(air, None, None, water)
    b_det = g.boundary(air, sens, sens, det)
    s0 = g.add_solid("world", [(box3(1200.0, 1200.0, 1200.0), b_world), (box3(1000.0, 1000.0, 1000.0), b_water)])
    s1 = g.add_solid("disc", [(cylinder(40.0, -0.05, 0.05), b_det)])
    g.add_instance(s0)
    k = 0
    wall = 600.0 - 0.05 - 0.01
    ticks = (np.arange(detectors_per_face) - (detectors_per_face - 1) / 2) * 250.0
    for axis, sign in ((0, 1), (0, -1), (1, 1), (1, -1)):
        inward = np.zeros(3)
        inward[axis] = -sign
        for a in ticks:
            for b in ticks:
                p = np.zeros(3)
                p[axis] = sign * wall
                other = [i for i in range(3) if i != axis]
                p[other[0]] = a
                p[other[1]] = b
                m = rotate_z_to(inward) @ translate(*p)
                g.add_instance(s1, m, sensor_identifier=k, sensor_index=k)
                k += 1
    g.icdf = default_icdf()
    g.water_boundary = b_water
    return g


def fibonacci_sphere(n, radius):
    i = np.arange(n, dtype=np.float64) + 0.5
    phi = np.arccos(1.0 - 2.0 * i / n)
    theta = math.pi * (1.0 + 5.0 ** 0.5) * i
    return radius * np.stack([np.cos(theta) * np.sin(phi), np.sin(theta) * np.sin(phi), np.cos(phi)], axis=1)


def large_sphere(num_sensors=20000, sphere_radius=17700.0, sensor_radius=19400.0, shell=120.0):
    """Acrylic sphere r=17.7 m holding liquid scintillator, 20,000 instanced sensors on r=19.4 m in water.

    Each sensor is a depth-3 union tree: ellipsoid (sphere r=254 scaled to 254,254,184), a body cylinder
    (r=127, h=200) and a neck cylinder (r=50, h=60), local +z facing the centre.  The ellipsoid's front cap is
    split into its own prim (z > 0 half of the ellipsoid, a zsphere scaled likewise) carrying the efficiency-0.3
    sensor surface, because the reference applies a surface to a whole prim.
    """
    g = Geometry("large_sphere")
    water = Material("Water", rindex=1.33, abslength=6e4, rayleigh=5e4)
    acrylic = Material("Acrylic", rindex=1.49, abslength=5e4)
    ls = Material("LS", rindex=1.48, abslength=7e4, rayleigh=2.7e4, reemprob=0.4)
    glass = Material("Glass", rindex=1.5, abslength=1e3)
    black = Surface.absorber("Blackened")
    sens = Surface.sensor("CapSensor", 0.3)
    world_r = sensor_radius + 1000.0
    b_world = g.boundary(water, None, black, water)
    b_acr = g.boundary(water, None, None, acrylic)
    b_ls = g.boundary(acrylic, None, None, ls)
    b_body = g.boundary(water, black, None, glass)
    b_cap = g.boundary(water, sens, None, glass)
    s0 = g.add_solid("world", [(sphere(world_r), b_world), (sphere(sphere_radius + shell), b_acr),
                               (sphere(sphere_radius), b_ls)])
    ell = with_transform(sphere(254.0), scale(1.0, 1.0, 184.0 / 254.0))
    body = with_transform(cylinder(127.0, -100.0, 100.0), translate(0, 0, -184.0))
    neck = with_transform(cylinder(50.0, -30.0, 30.0), translate(0, 0, -184.0 - 100.0 - 30.0 + 1.0))
    tree = operation(L.CSG_UNION, operation(L.CSG_UNION, ell, body), neck)
    cap = with_transform(zsphere(254.5, 0.0, 254.5), scale(1.0, 1.0, 184.5 / 254.5))
    s1 = g.add_solid("sensor", [(tree, b_body), (cap, b_cap)])
    g.add_instance(s0)
    pos = fibonacci_sphere(num_sensors, sensor_radius)
    for k, p in enumerate(pos):
        inward = -p / np.linalg.norm(p)
        m = rotate_z_to(inward) @ translate(*p)
        g.add_instance(s1, m, sensor_identifier=k, sensor_index=k)
    g.icdf = default_icdf()
    g.ls_boundary = b_ls
    return g
