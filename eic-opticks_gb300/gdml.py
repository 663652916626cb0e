"""Geant4-free loader for the GDML subset of the reference's detector descriptions.

The reference reads GDML through Geant4 (G4GDMLParser, g4cx/G4CXOpticks.cc:88-110) and translates the volume tree
(u4/U4Tree.h), solids (u4/U4Solid.h), materials (sysrap/sstandard.h) and surfaces (u4/U4SurfaceArray.h) into its
CSGFoundry and boundary arrays.  This module does the same translation straight from the XML into a
``geometry.Geometry``:

* defines: constant / variable / quantity, position, rotation, matrix (property tables);
* materials: optical property matrices (RINDEX, ABSLENGTH, RAYLEIGH, REEMISSIONPROB, GROUPVEL, FASTCOMPONENT or
  SCINTILLATIONCOMPONENT1); element composition is ignored (it does not enter the optical path);
* solids: box, orb, sphere (inner radius, theta range), ellipsoid (z cuts), tube (inner radius), cone (inner radii),
  polycone, union / subtraction / intersection with position and rotation of the second solid; trd and trap as
  convex polyhedra (beyond the reference, whose U4Solid has no G4Trd / G4Trap);
* opticalsurface + bordersurface / skinsurface;
* structure: volumes and physvol placements (position, rotation, positionref, rotationref), the setup's world.

Each placed volume becomes one instance of a one-prim solid (one solid per logical volume and boundary); its
boundary is (omat, osur, isur, imat) chosen as U4TreeBorder does, with the implicit perfect-absorber surfaces for
RINDEX -> no-RINDEX borders (u4/U4TreeBorder.h).  Expressions in attributes are evaluated by a small arithmetic
evaluator (numbers, + - * / ** and parentheses, defined constants, units, a few math functions); nothing in the
file is executed.
"""
import ast
import math
import operator
import xml.etree.ElementTree as ET

import numpy as np

from . import geometry as G
from . import layout as L

# CLHEP units, Geant4 internal system (mm, ns, MeV, rad)
UNITS = {
    "mm": 1.0, "millimeter": 1.0, "cm": 10.0, "centimeter": 10.0, "m": 1000.0, "meter": 1000.0, "km": 1e6,
    "um": 1e-3, "micrometer": 1e-3, "nm": 1e-6, "nanometer": 1e-6,
    "rad": 1.0, "radian": 1.0, "mrad": 1e-3, "deg": math.pi / 180.0, "degree": math.pi / 180.0,
    "ns": 1.0, "nanosecond": 1.0, "s": 1e9, "second": 1e9, "ms": 1e6, "us": 1e3, "ps": 1e-3,
    "MeV": 1.0, "eV": 1e-6, "keV": 1e-3, "GeV": 1e3,
    "pi": math.pi, "twopi": 2 * math.pi, "halfpi": math.pi / 2, "e": math.e,
    "g": 1.0, "mg": 1e-3, "kg": 1e3, "mole": 1.0, "K": 1.0, "kelvin": 1.0, "cm3": 1000.0, "m3": 1e9, "mm3": 1.0,
}
_FUNCS = {"sin": math.sin, "cos": math.cos, "tan": math.tan, "sqrt": math.sqrt, "exp": math.exp, "log": math.log,
          "abs": abs, "pow": math.pow, "asin": math.asin, "acos": math.acos, "atan": math.atan}
_BIN = {ast.Add: operator.add, ast.Sub: operator.sub, ast.Mult: operator.mul, ast.Div: operator.truediv,
        ast.Pow: operator.pow}
_UN = {ast.UAdd: operator.pos, ast.USub: operator.neg}
MEV_NM = 1239.8418754200e-6      # h c in MeV nm


class Expr:
    """Arithmetic over numbers, names (defined constants and units) and whitelisted math calls."""

    def __init__(self):
        self.names = dict(UNITS)

    def __call__(self, text):
        text = str(text).strip().replace("^", "**")
        return float(self._eval(ast.parse(text, mode="eval").body))

    def _eval(self, n):
        if isinstance(n, ast.Constant) and isinstance(n.value, (int, float)):
            return n.value
        if isinstance(n, ast.BinOp) and type(n.op) in _BIN:
            return _BIN[type(n.op)](self._eval(n.left), self._eval(n.right))
        if isinstance(n, ast.UnaryOp) and type(n.op) in _UN:
            return _UN[type(n.op)](self._eval(n.operand))
        if isinstance(n, ast.Name) and n.id in self.names:
            return self.names[n.id]
        if (isinstance(n, ast.Call) and isinstance(n.func, ast.Name) and n.func.id in _FUNCS and not n.keywords):
            return _FUNCS[n.func.id](*[self._eval(a) for a in n.args])
        raise ValueError("unsupported GDML expression element: %s" % ast.dump(n)[:80])


def _strip(tag):
    return tag.split("}", 1)[-1]


def _rot_matrix(ax, ay, az):
    """G4GDMLRead rotation: R = Rz Ry Rx (CLHEP rotateX, rotateY, rotateZ); the placement uses R^-1."""
    def rx(a):
        c, s = math.cos(a), math.sin(a)
        return np.array([[1, 0, 0], [0, c, -s], [0, s, c]])

    def ry(a):
        c, s = math.cos(a), math.sin(a)
        return np.array([[c, 0, s], [0, 1, 0], [-s, 0, c]])

    def rz(a):
        c, s = math.cos(a), math.sin(a)
        return np.array([[c, -s, 0], [s, c, 0], [0, 0, 1]])
    return rz(az) @ ry(ay) @ rx(ax)


def _placement(pos, rot):
    """Row-vector forward transform of G4Transform3D(R^-1, pos): p_mother = R^-1 p + pos, i.e. rows of R^T^-1 = R."""
    m = np.eye(4)
    m[:3, :3] = _rot_matrix(*rot)          # (R^-1)^T == R for a rotation
    m[3, :3] = pos
    return m


class GDML:
    """Parsed GDML document; ``geometry()`` translates it."""

    def __init__(self, source):
        root = ET.fromstring(source) if source.lstrip().startswith("<") else ET.parse(source).getroot()
        self.ex = Expr()
        self.positions, self.rotations, self.matrices = {}, {}, {}
        self.materials, self.solids, self.surfaces = {}, {}, {}
        self.volumes, self.border, self.skin = {}, [], {}
        self.world = None
        for sec in root:
            tag = _strip(sec.tag)
            if tag == "define":
                self._defines(sec)
            elif tag == "materials":
                self._materials(sec)
            elif tag == "solids":
                self._solids_section = sec
            elif tag == "structure":
                self._structure(sec)
            elif tag == "setup":
                for w in sec:
                    if _strip(w.tag) == "world":
                        self.world = w.get("ref")
        self._solid_elems = {}
        for el in getattr(self, "_solids_section", []):
            tag = _strip(el.tag)
            if tag == "opticalsurface":
                self.surfaces[el.get("name")] = self._opticalsurface(el)
            else:
                self._solid_elems[el.get("name")] = el
        if self.world is None:
            raise ValueError("GDML has no setup/world")

    # -- define ----------------------------------------------------------------------------------------------
    def _val(self, el, attr, default=0.0, unit=1.0):
        v = el.get(attr)
        return default if v is None else self.ex(v) * unit

    def _defines(self, sec):
        for el in sec:
            tag, name = _strip(el.tag), el.get("name")
            if tag in ("constant", "variable"):
                self.ex.names[name] = self.ex(el.get("value"))
            elif tag == "quantity":
                self.ex.names[name] = self.ex(el.get("value")) * UNITS.get(el.get("unit", ""), 1.0)
            elif tag == "position":
                u = UNITS[el.get("unit", "mm")]
                self.positions[name] = np.array([self._val(el, a, 0.0, u) for a in "xyz"])
            elif tag == "rotation":
                u = UNITS[el.get("unit", "rad")]
                self.rotations[name] = np.array([self._val(el, a, 0.0, u) for a in "xyz"])
            elif tag == "matrix":
                coldim = int(el.get("coldim", "1"))
                vals = np.array([self.ex(t) for t in el.get("values", "").split()], dtype=np.float64)
                self.matrices[name] = vals.reshape(-1, coldim)
                if coldim == 1 and len(vals) == 1:
                    self.ex.names[name] = vals[0]

    # -- materials -------------------------------------------------------------------------------------------
    def _materials(self, sec):
        for el in sec:
            if _strip(el.tag) != "material":
                continue
            props = {}
            for p in el:
                if _strip(p.tag) == "property":
                    ref = p.get("ref")
                    if ref in self.matrices and self.matrices[ref].shape[1] == 2:
                        props[p.get("name")] = self.matrices[ref]
            self.materials[el.get("name")] = props

    @staticmethod
    def _on_domain(table, default):
        """Property table (energy in MeV, value) sampled at the 761 domain wavelengths by linear interpolation in
        energy, edge values outside the table (G4PhysicsVector::Value)."""
        if table is None:
            return lambda wl: np.full(np.shape(wl), float(default))
        e = table[:, 0]
        v = table[:, 1]
        order = np.argsort(e)
        e, v = e[order], v[order]
        return lambda wl: np.interp(MEV_NM / np.asarray(wl, dtype=np.float64), e, v)

    def _material(self, name):
        props = self.materials.get(name, {})
        gv = props.get("GROUPVEL")
        return G.Material(name, rindex=self._on_domain(props.get("RINDEX"), 1.0),
                          abslength=self._on_domain(props.get("ABSLENGTH"), 1e12),
                          rayleigh=self._on_domain(props.get("RAYLEIGH"), 1e12),
                          reemprob=self._on_domain(props.get("REEMISSIONPROB"), 0.0),
                          groupvel=None if gv is None else self._on_domain(gv, G.C_LIGHT))

    def has_rindex(self, material):
        return "RINDEX" in self.materials.get(material, {})

    # -- surfaces --------------------------------------------------------------------------------------------
    _FINISH = {"polished": 0, "polishedfrontpainted": 1, "polishedbackpainted": 2, "ground": 3,
               "groundfrontpainted": 4, "groundbackpainted": 5}

    def _opticalsurface(self, el):
        fin = el.get("finish", "0")
        finish = int(self.ex(fin)) if fin not in self._FINISH else self._FINISH[fin]
        props = {}
        for p in el:
            if _strip(p.tag) == "property" and p.get("ref") in self.matrices:
                props[p.get("name")] = self.matrices[p.get("ref")]
        return dict(name=el.get("name"), finish=finish, value=self.ex(el.get("value", "1")), props=props)

    def _surface(self, osname, label):
        """U4SurfaceArray::addSurface: sensor if any EFFICIENCY > 0 on the domain (detect / absorb), else polished
        finishes reflect specularly and the others diffusely with REFLECTIVITY (absent -> 0)."""
        os_ = self.surfaces[osname]
        effi = self._on_domain(os_["props"].get("EFFICIENCY"), 0.0)(G.DOMAIN)
        refl = self._on_domain(os_["props"].get("REFLECTIVITY"), 0.0)(G.DOMAIN)
        ems = {"@": L.EMS_SURFACE_ZPLUS_CUSTOMART, "#": L.EMS_SURFACE_ZPLUS_A, "!": L.EMS_SURFACE_ZMINUS}.get(
            os_["name"][:1], L.EMS_SURFACE) if hasattr(L, "EMS_SURFACE_ZPLUS_A") else L.EMS_SURFACE
        common = dict(ems=ems, finish=os_["finish"], value_percent=int(100.0 * os_["value"]))
        if effi.max() > 0.0:
            return G.Surface(label, detect=effi, absorb=1.0 - effi, **common)
        if os_["finish"] in (0, 1, 2):
            return G.Surface(label, absorb=1.0 - refl, specular=refl, **common)
        return G.Surface(label, absorb=1.0 - refl, diffuse=refl, **common)

    # -- solids ----------------------------------------------------------------------------------------------
    def solid(self, name):
        if name not in self.solids:
            self.solids[name] = self._solid(self._solid_elems[name])
        return self.solids[name]

    def _solid(self, el):
        tag = _strip(el.tag)
        lu = UNITS[el.get("lunit", "mm")]
        au = UNITS[el.get("aunit", "rad")]
        v = lambda a, d=0.0: self._val(el, a, d, lu)          # noqa: E731
        if tag == "box":
            return G.box3(v("x"), v("y"), v("z"))
        if tag == "orb":
            return G.sphere(v("r"))
        if tag == "sphere":
            return self._sphere(v("rmin"), v("rmax"), self._val(el, "starttheta", 0.0, au),
                                self._val(el, "deltatheta", math.pi, au), self._val(el, "startphi", 0.0, au),
                                self._val(el, "deltaphi", 2 * math.pi, au))
        if tag == "ellipsoid":
            return self._ellipsoid(v("ax"), v("by"), v("cz"), el.get("zcut1"), el.get("zcut2"), lu)
        if tag == "tube":
            return self._tube(v("rmin"), v("rmax"), v("z") / 2)
        if tag == "cone":
            return self._cone(v("rmin1"), v("rmax1"), v("rmin2"), v("rmax2"), v("z") / 2)
        if tag == "polycone":
            planes = [(self._val(z, "rmin", 0.0, lu), self._val(z, "rmax", 0.0, lu), self._val(z, "z", 0.0, lu))
                      for z in el if _strip(z.tag) == "zplane"]
            return self._polycone(planes)
        if tag == "trd":
            hx1, hx2, hy1, hy2, hz = v("x1") / 2, v("x2") / 2, v("y1") / 2, v("y2") / 2, v("z") / 2
            return self._hull([(sx * hx, sy * hy, z) for z, hx, hy in ((-hz, hx1, hy1), (hz, hx2, hy2))
                               for sx in (-1, 1) for sy in (-1, 1)])
        if tag == "trap":
            return self._trap(v("z") / 2, self._val(el, "theta", 0.0, au), self._val(el, "phi", 0.0, au),
                              v("y1") / 2, v("x1") / 2, v("x2") / 2, self._val(el, "alpha1", 0.0, au),
                              v("y2") / 2, v("x3") / 2, v("x4") / 2, self._val(el, "alpha2", 0.0, au))
        if tag in ("union", "subtraction", "intersection"):
            first = second = None
            pos, rot = np.zeros(3), np.zeros(3)
            for c in el:
                ct = _strip(c.tag)
                if ct == "first":
                    first = self.solid(c.get("ref"))
                elif ct == "second":
                    second = self.solid(c.get("ref"))
                elif ct == "position":
                    u = UNITS[c.get("unit", "mm")]
                    pos = np.array([self._val(c, a, 0.0, u) for a in "xyz"])
                elif ct == "positionref":
                    pos = self.positions[c.get("ref")]
                elif ct == "rotation":
                    u = UNITS[c.get("unit", "rad")]
                    rot = np.array([self._val(c, a, 0.0, u) for a in "xyz"])
                elif ct == "rotationref":
                    rot = self.rotations[c.get("ref")]
                elif ct in ("firstposition", "firstrotation", "firstpositionref", "firstrotationref"):
                    raise ValueError("GDML boolean %s: first-solid placement is not supported" % el.get("name"))
            if np.any(pos) or np.any(rot):
                second = _place(second, _placement(pos, rot))
            op = {"union": L.CSG_UNION, "subtraction": L.CSG_DIFFERENCE, "intersection": L.CSG_INTERSECTION}[tag]
            return G.operation(op, first, second)
        raise ValueError("GDML solid <%s> (%s) is not supported" % (tag, el.get("name")))

    @staticmethod
    def _sphere(rmin, rmax, theta0, dtheta, phi0, dphi):
        if phi0 != 0.0 or abs(dphi - 2 * math.pi) > 1e-12:
            raise ValueError("sphere with a phi segment is not supported (u4/U4Solid.h init_Sphere_)")

        def layer(r):
            if r == 0.0:
                return None
            zmin, zmax = r * math.cos(theta0 + dtheta), r * math.cos(theta0)
            return G.zsphere(r, zmin, zmax) if (theta0 > 0.0 or dtheta < math.pi) else G.sphere(r)
        outer, inner = layer(rmax), layer(rmin)
        return outer if inner is None else G.operation(L.CSG_DIFFERENCE, outer, inner)

    def _ellipsoid(self, ax, by, cz, zcut1, zcut2, lu):
        """U4Solid::init_Ellipsoid: a sphere of radius cz scaled (ax/cz, by/cz, 1), z cuts as a zsphere with the
        0.1 mm safety on an uncut end."""
        zmin = max(self.ex(zcut1) * lu, -cz) if zcut1 is not None else -cz
        zmax = min(self.ex(zcut2) * lu, cz) if zcut2 is not None else cz
        lower, upper = zmin > -cz, zmax < cz
        if not lower and not upper:
            nd = G.sphere(cz)
        elif lower and upper:
            nd = G.zsphere(cz, zmin, zmax)
        elif lower:
            nd = G.zsphere(cz, zmin, zmax + 0.1)
        else:
            nd = G.zsphere(cz, zmin - 0.1, zmax)
        return G.with_transform(nd, G.scale(ax / cz, by / cz, 1.0))

    @staticmethod
    def _tube(rmin, rmax, hz):
        """U4Solid::init_Tubs: cylinder, minus an inner cylinder 1 % longer when rmin > 0 (phi ignored, as there)."""
        outer = G.cylinder(rmax, -hz, hz)
        if rmin <= 0.0:
            return outer
        dz = hz * 0.01
        return G.operation(L.CSG_DIFFERENCE, outer, G.cylinder(rmin, -(hz + dz), hz + dz))

    @staticmethod
    def _cone(rmin1, rmax1, rmin2, rmax2, hz):
        outer = G.cone(rmax1, -hz, rmax2, hz)
        if rmin1 == 0.0 and rmin2 == 0.0:
            return outer
        return G.operation(L.CSG_DIFFERENCE, outer, G.cone(rmin1, -hz, rmin2, hz))

    @staticmethod
    def _union_tree(items):
        while len(items) > 1:
            nxt = [G.operation(L.CSG_UNION, items[i], items[i + 1]) for i in range(0, len(items) - 1, 2)]
            if len(items) % 2:
                nxt.append(items[-1])
            items = nxt
        return items[0]

    def _polycone(self, planes):
        """Union of the z sections (a cylinder where both radii agree, else a cone), minus the same built from the
        inner radii when any is non-zero (u4/U4Polycone.h)."""
        planes = sorted(planes, key=lambda p: p[2])

        def sections(k):
            out = []
            for (a, b) in zip(planes[:-1], planes[1:]):
                r1, r2, z1, z2 = a[k], b[k], a[2], b[2]
                if z2 <= z1 or (r1 == 0.0 and r2 == 0.0):
                    continue
                out.append(G.cylinder(r1, z1, z2) if r1 == r2 else G.cone(r1, z1, r2, z2))
            return out
        outer = self._union_tree(sections(1))
        inner = sections(0)
        return outer if not inner else G.operation(L.CSG_DIFFERENCE, outer, self._union_tree(inner))

    @staticmethod
    def _hull(verts):
        """Convex polyhedron of 8 vertices ordered (z0: --, -+, +-, ++; z1: same): six face planes."""
        p = np.asarray(verts, dtype=np.float64)
        faces = [(0, 1, 3, 2), (4, 6, 7, 5), (0, 4, 5, 1), (2, 3, 7, 6), (0, 2, 6, 4), (1, 5, 7, 3)]
        centre = p.mean(axis=0)
        planes = []
        for f in faces:
            a, b, c = p[f[0]], p[f[1]], p[f[2]]
            n = np.cross(b - a, c - a)
            if np.linalg.norm(n) < 1e-12:
                a, b, c = p[f[0]], p[f[2]], p[f[3]]
                n = np.cross(b - a, c - a)
            n /= np.linalg.norm(n)
            if np.dot(n, a - centre) < 0:
                n = -n
            planes.append((*n, float(np.dot(n, a))))
        lo, hi = p.min(axis=0), p.max(axis=0)
        return G.convexpolyhedron(planes, (*lo, *hi))

    def _trap(self, dz, theta, phi, dy1, dx1, dx2, alp1, dy2, dx3, dx4, alp2):
        """G4Trap vertices (G4Trap::MakePlanes corner formulae)."""
        tt = math.tan(theta)
        tcp, tsp = tt * math.cos(phi), tt * math.sin(phi)
        ta1, ta2 = math.tan(alp1), math.tan(alp2)
        v = [(-dz * tcp - dy1 * ta1 - dx1, -dz * tsp - dy1, -dz), (-dz * tcp - dy1 * ta1 + dx1, -dz * tsp - dy1, -dz),
             (-dz * tcp + dy1 * ta1 - dx2, -dz * tsp + dy1, -dz), (-dz * tcp + dy1 * ta1 + dx2, -dz * tsp + dy1, -dz),
             (dz * tcp - dy2 * ta2 - dx3, dz * tsp - dy2, dz), (dz * tcp - dy2 * ta2 + dx3, dz * tsp - dy2, dz),
             (dz * tcp + dy2 * ta2 - dx4, dz * tsp + dy2, dz), (dz * tcp + dy2 * ta2 + dx4, dz * tsp + dy2, dz)]
        # reorder to (z0: --, -+, +-, ++) in (x, y): corners 0,2,1,3 of each face
        return self._hull([v[0], v[2], v[1], v[3], v[4], v[6], v[5], v[7]])

    # -- structure -------------------------------------------------------------------------------------------
    def _structure(self, sec):
        for el in sec:
            tag = _strip(el.tag)
            if tag == "volume":
                vol = dict(material=None, solid=None, physvols=[], aux={})
                self._volume_children(el, vol, {})
                self.volumes[el.get("name")] = vol
            elif tag == "bordersurface":
                pvs = [c.get("ref") for c in el if _strip(c.tag) == "physvolref"]
                self.border.append((pvs[0], pvs[1], el.get("surfaceproperty"), el.get("name")))
            elif tag == "skinsurface":
                lv = [c.get("ref") for c in el if _strip(c.tag) == "volumeref"][0]
                self.skin[lv] = (el.get("surfaceproperty"), el.get("name"))

    def _volume_children(self, el, vol, loopvars):
        """Children of a <volume>, with <loop for= from= to= step=> expanded: the loop variable is defined while
        its body is read and "{var}" in physvol names takes its integer value (G4GDMLRead::LoopRead)."""
        for c in el:
            ct = _strip(c.tag)
            if ct == "materialref":
                vol["material"] = c.get("ref")
            elif ct == "solidref":
                vol["solid"] = c.get("ref")
            elif ct == "auxiliary":
                vol["aux"][c.get("auxtype")] = c.get("auxvalue")
            elif ct == "physvol":
                pv = self._physvol(c)
                for var, val in loopvars.items():
                    pv["name"] = pv["name"].replace("{%s}" % var, "%d" % val)
                vol["physvols"].append(pv)
            elif ct == "loop":
                var = c.get("for")
                lo, hi, step = self.ex(c.get("from")), self.ex(c.get("to")), self.ex(c.get("step", "1"))
                if step <= 0 or (hi - lo) / step > 1e6:
                    raise ValueError("GDML loop over %s: bad range" % var)
                saved = self.ex.names.get(var)
                x = lo
                while x <= hi + 1e-9:
                    self.ex.names[var] = x
                    self._volume_children(c, vol, dict(loopvars, **{var: int(round(x))}))
                    x += step
                if saved is None:
                    self.ex.names.pop(var, None)
                else:
                    self.ex.names[var] = saved

    def _physvol(self, el):
        pv = dict(name=el.get("name"), volume=None, pos=np.zeros(3), rot=np.zeros(3),
                  copyno=int(el.get("copynumber", "0")))
        for c in el:
            ct = _strip(c.tag)
            if ct == "volumeref":
                pv["volume"] = c.get("ref")
            elif ct == "position":
                u = UNITS[c.get("unit", "mm")]
                pv["pos"] = np.array([self._val(c, a, 0.0, u) for a in "xyz"])
            elif ct == "positionref":
                pv["pos"] = self.positions[c.get("ref")]
            elif ct == "rotation":
                u = UNITS[c.get("unit", "rad")]
                pv["rot"] = np.array([self._val(c, a, 0.0, u) for a in "xyz"])
            elif ct == "rotationref":
                pv["rot"] = self.rotations[c.get("ref")]
            elif ct in ("scale", "scaleref"):
                raise ValueError("physvol %s: reflected placements are not supported" % pv["name"])
        if pv["name"] is None:
            pv["name"] = "%s_pv" % pv["volume"]
        return pv

    def _find_surface(self, pre, post, pre_lv, post_lv, entering):
        """U4Surface::Find: border surface (pre -> post), else the skin surfaces, daughter's first when entering."""
        if pre is None or post is None:
            return None
        for a, b, prop, name in self.border:
            if a == pre and b == post:
                return prop, name
        order = (post_lv, pre_lv) if entering else (pre_lv, post_lv)
        for lv in order:
            if lv in self.skin:
                return self.skin[lv]
        return None

    # -- translation -----------------------------------------------------------------------------------------
    def geometry(self, name="gdml"):
        g = G.Geometry(name)
        self.placements = []                    # (pv name, lv, boundary, instance index)
        solid_cache = {}
        surf_cache = {}

        def surf(found):
            if found is None:
                return None
            prop, label = found
            if label not in surf_cache:
                surf_cache[label] = self._surface(prop, label)
            return surf_cache[label]

        def implicit(inner_pv, outer_pv, flip):
            label = "Implicit_RINDEX_NoRINDEX_%s_%s" % ((outer_pv, inner_pv) if flip else (inner_pv, outer_pv))
            if label not in surf_cache:
                surf_cache[label] = G.Surface(label, absorb=1.0, ems=L.EMS_SURFACE, finish=1, value_percent=100)
            return surf_cache[label]

        sensors = 0
        # the world's own physical volume (G4GDML places the world LV unnamed in the file): daughters of the world
        # look up surfaces against it, the world itself has no mother and so no surfaces (U4Surface::Find)
        stack = [(self.world + "_PV", self.world, None, None, np.eye(4))]
        while stack:
            pv, lv, parent_pv, parent_lv, m = stack.pop()
            vol = self.volumes[lv]
            imat = vol["material"]
            omat = self.volumes[parent_lv]["material"] if parent_lv is not None else imat
            osur = surf(self._find_surface(parent_pv, pv, parent_lv, lv, True))
            isur = surf(self._find_surface(pv, parent_pv, lv, parent_lv, False)) if self.has_rindex(imat) else None
            o_r, i_r = self.has_rindex(omat), self.has_rindex(imat)
            if parent_lv is not None:
                if osur is None and o_r and not i_r:
                    osur = implicit(pv, parent_pv, True)
                if isur is None and i_r and not o_r:
                    isur = implicit(pv, parent_pv, False)
            b = g.boundary(self._material(omat), osur, isur, self._material(imat))
            key = (lv, b)
            if key not in solid_cache:
                solid_cache[key] = g.add_solid(lv[:16], [(self.solid(vol["solid"]), b)])
            is_sensor = any(s is not None and float(np.max(s.detect)) > 0.0 for s in (osur, isur))
            sid = sensors if is_sensor else -1
            sensors += int(is_sensor)
            inst = g.add_instance(solid_cache[key], m if parent_lv is not None else None, sensor_identifier=sid,
                                  sensor_index=sid)
            self.placements.append((pv, lv, b, inst))
            for child in reversed(vol["physvols"]):
                stack.append((child["name"], child["volume"], pv, lv, _placement(child["pos"], child["rot"]) @ m))
        emission = None
        for mname, props in self.materials.items():
            comp = props.get("FASTCOMPONENT", props.get("SCINTILLATIONCOMPONENT1"))
            if comp is not None:
                order = np.argsort(comp[:, 0])
                emission = (comp[order, 0] * 1e6, comp[order, 1])       # MeV -> eV
                break
        if emission is not None:
            g.icdf = G.scint_icdf_table(*emission)
        return g


def _place(node, m):
    """Apply a row-vector placement to a CSG subtree (leaves carry the combined transform)."""
    if "left" in node:
        return G.operation(node["typecode"], _place(node["left"], m), _place(node["right"], m))
    return G.with_transform(node, m)


def load(source, name=None):
    """GDML file path or XML text -> (geometry.Geometry, GDML document)."""
    doc = GDML(source)
    return doc.geometry(name or doc.world), doc
