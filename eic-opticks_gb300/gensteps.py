"""Genstep and input-photon producers for the benchmark workloads.

In the reference, Geant4 process hooks pack ``quad6`` gensteps (u4/U4.cc:82-305) and the application can inject
photons directly (``SEvt::SetInputPhoton``, src/GPUPhotonSourceMinimal.h:59-87).  Geant4 is outside the hot
path, so these functions synthesise gensteps with the same field layout from seeded numpy generators:

* torch       sysrap/storch.h:43-69
* scintillation sysrap/sscint.h:34-62
* Cerenkov    sysrap/scerenkov.h:29-58, photon yield from the Frank-Tamm relation
* input photon  one INPUT_PHOTON genstep whose numphoton covers the supplied sphoton array
"""
import math
import numpy as np

from . import layout as L
from . import geometry as G

FINE_STRUCTURE_OVER_HBARC = 369.81   # photons / (eV cm) for unit charge (alpha / hbar c)


def _gs(n):
    return np.zeros((n, 6, 4), dtype=np.float32)


def _ints(g):
    return g.view(np.int32)


def input_photon_genstep(num_photon):
    g = _gs(1)
    gi = _ints(g)
    gi[0, 0, 0] = L.GS_INPUT_PHOTON
    g.view(np.uint32)[0, 0, 3] = num_photon
    return g


def isotropic_photons(n, wavelength=420.0, seed=42, origin=(0.0, 0.0, 0.0)):
    """Photons at ``origin``, isotropic direction, linear polarisation uniform in the transverse plane, t0=0."""
    rng = np.random.default_rng(seed)
    cost = rng.uniform(-1.0, 1.0, n)
    phi = rng.uniform(0.0, 2 * math.pi, n)
    sint = np.sqrt(1.0 - cost * cost)
    mom = np.stack([sint * np.cos(phi), sint * np.sin(phi), cost], axis=1)
    a = np.where(np.abs(mom[:, 2:3]) < 0.9, np.array([[0.0, 0.0, 1.0]]), np.array([[1.0, 0.0, 0.0]]))
    e1 = np.cross(a, mom)
    e1 /= np.linalg.norm(e1, axis=1, keepdims=True)
    e2 = np.cross(mom, e1)
    psi = rng.uniform(0.0, 2 * math.pi, n)[:, None]
    pol = np.cos(psi) * e1 + np.sin(psi) * e2
    p = np.zeros(n, dtype=L.PHOTON)
    p["pos"] = origin
    p["time"] = 0.0
    p["mom"] = mom.astype(np.float32)
    p["pol"] = pol.astype(np.float32)
    p["wavelength"] = wavelength
    return p


_FLT_MAX = np.finfo(np.float32).max


def _round_to_float32(frac):
    """The binary32 value nearest to an exact rational, ties to even (one rounding, as strtof does; a conversion
    through a Python float would round twice).  None when the value rounds beyond the binary32 range."""
    from fractions import Fraction
    lim = Fraction(int(_FLT_MAX)) + Fraction(2) ** 103          # half an ulp above the largest finite binary32
    if abs(frac) >= lim:
        return None
    c = np.float32(float(frac))
    best = None
    for cand in (np.nextafter(c, np.float32(-np.inf)), c, np.nextafter(c, np.float32(np.inf))):
        if not np.isfinite(cand):
            continue
        err = abs(Fraction(float(cand)) - frac)
        even = (int(np.array(cand, dtype=np.float32).view(np.uint32)) & 1) == 0
        if best is None or err < best[0] or (err == best[0] and even):
            best = (err, cand)
    return best[1]


def _cxx_extract_floats(line, count):
    """Reads `count` floats from a line the way ``std::istringstream >> float`` does in libstdc++'s "C" locale
    (num_get::_M_extract_float then strtof): skip white space, accumulate an optional sign, digits with at most one
    decimal point, and an exponent marker (only after a mantissa digit) with an optional sign and digits; the whole
    accumulation must convert, and a value beyond the binary32 range fails.  A failed extraction ends the line
    (returns None); what follows the last value is ignored.  So "nan", "inf", "1_0" (as a non-final value) and "1e"
    fail, "1_0" as the final value reads 1, and "1.5.5" reads 1.5 then .5."""
    from fractions import Fraction
    vals, i, n = [], 0, len(line)
    for _ in range(count):
        while i < n and line[i] in " \t\n\v\f\r":
            i += 1
        acc = ""
        if i < n and line[i] in "+-":
            acc += line[i]
            i += 1
        found_mant = found_dec = found_sci = False
        while i < n:
            c = line[i]
            if c.isdigit() and c in "0123456789":
                acc += c
                found_mant = True
            elif c == "." and not found_dec and not found_sci:
                acc += c
                found_dec = True
            elif c in "eE" and not found_sci and found_mant:
                acc += "e"
                found_sci = True
                i += 1
                if i < n and line[i] in "+-":
                    acc += line[i]
                else:
                    continue
            else:
                break
            i += 1
        mant = acc.split("e")[0].lstrip("+-")
        expo = acc.split("e")[1] if "e" in acc else None
        if not any(ch.isdigit() for ch in mant) or (expo is not None and not expo.lstrip("+-")):
            return None
        v = _round_to_float32(Fraction(acc))
        if v is None:
            return None
        vals.append(v)
    return vals


def load_photons_txt(path):
    """Input photons from a text file as the reference's photon-file source reads them (src/GPUPhotonFileSource.h
    load_photons_txt): one photon per line, 11 values ``pos_x pos_y pos_z time mom_x mom_y mom_z pol_x pol_y pol_z
    wavelength`` read by C++ stream extraction (see _cxx_extract_floats); blank lines and lines starting with '#'
    skipped, lines whose 11 extractions do not all succeed skipped, anything after the 11th value ignored.  Other
    fields are zero."""
    rows = []
    with open(path, "rb") as f:
        text = f.read().decode("latin-1")        # bytes as std::getline sees them; lines end at '\n' only
    for line in text.split("\n"):
        if not line or line[0] == "#":
            continue
        v = _cxx_extract_floats(line, 11)
        if v is not None:
            rows.append(v)
    p = np.zeros(len(rows), dtype=L.PHOTON)
    if rows:
        a = np.asarray(rows, dtype=np.float32)
        p["pos"] = a[:, 0:3]
        p["time"] = a[:, 3]
        p["mom"] = a[:, 4:7]
        p["pol"] = a[:, 7:10]
        p["wavelength"] = a[:, 10]
    return p


def _g(x):
    """A number as C++ iostream writes a double by default (6 significant digits, %g)."""
    return "%g" % float(x)


def write_hits_txt(hits, path):
    """Hits in the text format of the reference's photon-file application (src/GPUPhotonFileSource.h
    EndOfEventAction): ``time wavelength  (x, y, z)  (mx, my, mz)  (px, py, pz)`` per line."""
    with open(path, "w") as f:
        for h in hits:
            pos, mom, pol = h["pos"], h["mom"], h["pol"]
            f.write("%s %s  (%s, %s, %s)  (%s, %s, %s)  (%s, %s, %s)\n" % (
                _g(h["time"]), _g(h["wavelength"]), _g(pos[0]), _g(pos[1]), _g(pos[2]),
                _g(mom[0]), _g(mom[1]), _g(mom[2]), _g(pol[0]), _g(pol[1]), _g(pol[2])))


TORCH_TYPES = {"disc": L.T_DISC, "line": L.T_LINE, "point": L.T_POINT, "circle": L.T_CIRCLE,
               "rectangle": L.T_RECTANGLE, "sphere_marsaglia": L.T_SPHERE_MARSAGLIA, "sphere": L.T_SPHERE}


def torch_genstep_from_config(path):
    """The torch genstep and event settings of a reference application config file (config/*.json, read by
    gphox::Config::ReadConfig, src/config.cpp): ``torch`` gives every storch field (gentype, trackid, matline,
    numphoton, pos, time, mom (normalized in binary32), weight, pol, wavelength, zenith, azimuth, radius, distance,
    mode, type by name), ``event`` the event mode and maxslot.  Returns (gensteps (1,6,4) float32, event dict)."""
    import json
    with open(path) as f:
        cfg = json.load(f)
    t = cfg["torch"]
    if t.get("gentype", "TORCH") != "TORCH":
        raise ValueError("torch.gentype %r is not TORCH" % t.get("gentype"))
    if t["type"] not in TORCH_TYPES:
        raise ValueError("torch.type %r is not a torch type" % t["type"])
    g = torch_gensteps(1, int(t["numphoton"]), torch_type=TORCH_TYPES[t["type"]], pos=tuple(t["pos"]),
                       mom=tuple(t["mom"]), wavelength=float(t["wavelength"]), radius=float(t["radius"]),
                       zenith=tuple(t["zenith"]), azimuth=tuple(t["azimuth"]), distance=float(t["distance"]),
                       time=float(t["time"]))
    gu = g.view(np.uint32)
    gu[0, 0, 1] = int(t.get("trackid", 0))
    gu[0, 0, 2] = int(t.get("matline", 0))
    g[0, 2, 3] = float(t.get("weight", 0.0))
    g[0, 3, 0:3] = t.get("pol", (0.0, 0.0, 0.0))
    gu[0, 5, 2] = int(t.get("mode", 255))
    ev = cfg.get("event", {})
    return g, {"mode": ev.get("mode"), "maxslot": ev.get("maxslot")}


def torch_gensteps(num_gs, photons_per_gs, torch_type=L.T_DISC, pos=(0.0, 0.0, -90.0), mom=(0.0, 0.0, 1.0),
                   wavelength=420.0, radius=50.0, zenith=(0.0, 1.0), azimuth=(0.0, 1.0), distance=0.0, time=0.0):
    """Torch gensteps with storch.h fields: pos/time, mom/weight, pol/wavelength, zenith, azimuth,
    radius/distance/mode/type (storch::FillGenstep defaults, sysrap/storch.h:86-150)."""
    g = _gs(num_gs)
    gu = g.view(np.uint32)
    gu[:, 0, 0] = L.GS_TORCH
    gu[:, 0, 3] = photons_per_gs
    m = np.asarray(mom, dtype=np.float32)
    dot = np.float32(m[0] * m[0]) + np.float32(m[1] * m[1]) + np.float32(m[2] * m[2])
    m = m * (np.float32(1.0) / np.sqrt(np.float32(dot)))       # normalize(float3), sysrap/scuda.h:606-610
    g[:, 1, 0:3] = pos
    g[:, 1, 3] = time
    g[:, 2, 0:3] = m
    g[:, 2, 3] = 0.0                    # weight (FillGenstep default "0")
    g[:, 3, 3] = wavelength
    g[:, 4, 0:2] = zenith
    g[:, 4, 2:4] = azimuth
    g[:, 5, 0] = radius
    g[:, 5, 1] = distance
    gu[:, 5, 2] = 255                   # mode (FillGenstep sets 255)
    gu[:, 5, 3] = torch_type
    return g


def crystal_scint_gensteps(num_gs=2000, mean_photons=5000, seed=42, n=8, scint_time=1000.0, poisson=True):
    """Scintillation deposits in the 8x8 crystal array.

    Position: a random crystal, x/y uniform over its cross-section (1 mm from the walls), depth below the front
    face exponential with 50 mm scale (resampled to stay 5 mm clear of the back face), isotropic 1 mm step.
    numphoton ~ Poisson(mean_photons); charge 0 so the reference skips the step-fraction draw (qscint.h:66).
    """
    rng = np.random.default_rng(seed)
    g = _gs(num_gs)
    gu = g.view(np.uint32)
    gu[:, 0, 0] = L.GS_SCINTILLATION
    gu[:, 0, 1] = np.arange(num_gs)
    gu[:, 0, 2] = 0
    cnt = rng.poisson(mean_photons, num_gs) if poisson else np.full(num_gs, mean_photons)
    gu[:, 0, 3] = cnt
    ci = rng.integers(0, n, num_gs)
    cj = rng.integers(0, n, num_gs)
    cx = (ci - (n - 1) / 2) * G.CRYSTAL_PITCH
    cy = (cj - (n - 1) / 2) * G.CRYSTAL_PITCH
    x = cx + rng.uniform(-9.0, 9.0, num_gs)
    y = cy + rng.uniform(-9.0, 9.0, num_gs)
    depth = rng.exponential(50.0, num_gs)
    while True:
        bad = depth > 194.0
        if not bad.any():
            break
        depth[bad] = rng.exponential(50.0, bad.sum())
    z = -100.0 + 1.0 + depth
    cost = rng.uniform(-1, 1, num_gs)
    phi = rng.uniform(0, 2 * math.pi, num_gs)
    sint = np.sqrt(1 - cost * cost)
    step = 1.0
    d = np.stack([sint * np.cos(phi), sint * np.sin(phi), cost], axis=1) * step
    g[:, 1, 0] = x
    g[:, 1, 1] = y
    g[:, 1, 2] = z
    g[:, 1, 3] = 0.0
    g[:, 2, 0:3] = d
    g[:, 2, 3] = step
    _ints(g)[:, 3, 0] = 0          # code
    g[:, 3, 1] = 0.0               # charge
    g[:, 3, 2] = 1.0               # weight
    g[:, 3, 3] = 0.9 * G.C_LIGHT   # meanVelocity
    g[:, 5, 0] = scint_time
    return g


def sphere_scint_gensteps(num_gs, mean_photons, seed=42, radius=17000.0, scint_time=10.0, poisson=False):
    """Scintillation deposits uniform within r < radius (large-sphere workload)."""
    rng = np.random.default_rng(seed)
    g = _gs(num_gs)
    gu = g.view(np.uint32)
    gu[:, 0, 0] = L.GS_SCINTILLATION
    gu[:, 0, 1] = np.arange(num_gs)
    gu[:, 0, 3] = rng.poisson(mean_photons, num_gs) if poisson else mean_photons
    u = rng.uniform(0, 1, num_gs) ** (1.0 / 3.0) * radius
    cost = rng.uniform(-1, 1, num_gs)
    phi = rng.uniform(0, 2 * math.pi, num_gs)
    sint = np.sqrt(1 - cost * cost)
    g[:, 1, 0] = u * sint * np.cos(phi)
    g[:, 1, 1] = u * sint * np.sin(phi)
    g[:, 1, 2] = u * cost
    g[:, 2, 0:3] = (0.0, 0.0, 1.0)
    g[:, 2, 3] = 1.0
    g[:, 3, 2] = 1.0
    g[:, 3, 3] = 0.9 * G.C_LIGHT
    g[:, 5, 0] = scint_time
    return g


def frank_tamm_mean_photons(beta, rindex_table, step_mm, charge=1.0):
    """Mean Cerenkov photons for a step: (alpha z^2 / hbar c) * step * integral (1 - 1/(beta n)^2) dE."""
    wl = rindex_table[:, 0]
    n = rindex_table[:, 1]
    e = G.HC_EVNM / wl
    order = np.argsort(e)
    e, n = e[order], n[order]
    integrand = np.clip(1.0 - 1.0 / (beta * beta * n * n), 0.0, None)
    integral = float(np.sum(0.5 * (integrand[1:] + integrand[:-1]) * np.diff(e)))
    return FINE_STRUCTURE_OVER_HBARC * charge * charge * integral * (step_mm / 10.0)


def water_cerenkov_gensteps(geom, num_gs=1000, seed=42, step=2.0, half=500.0, margin=5.0):
    """Charged-track steps in the water cube: start uniform in the water, direction isotropic, beta ~ U[0.8, 1]."""
    rng = np.random.default_rng(seed)
    table = G.water_refractive_index_table()
    nmax = float(table[:, 1].max())
    g = _gs(num_gs)
    gu = g.view(np.uint32)
    gu[:, 0, 0] = L.GS_CERENKOV
    gu[:, 0, 1] = np.arange(num_gs)
    gu[:, 0, 2] = geom.material_line(geom.water_boundary)
    lim = half - margin
    pos = rng.uniform(-lim, lim, (num_gs, 3))
    cost = rng.uniform(-1, 1, num_gs)
    phi = rng.uniform(0, 2 * math.pi, num_gs)
    sint = np.sqrt(1 - cost * cost)
    d = np.stack([sint * np.cos(phi), sint * np.sin(phi), cost], axis=1) * step
    beta = rng.uniform(0.8, 1.0, num_gs)
    # Frank-Tamm yield for every step at once (same integral as frank_tamm_mean_photons)
    wl, n = table[:, 0], table[:, 1]
    e = G.HC_EVNM / wl
    order = np.argsort(e)
    e, n = e[order], n[order]
    integrand = np.clip(1.0 - 1.0 / (beta[:, None] ** 2 * n[None, :] ** 2), 0.0, None)
    integral = np.sum(0.5 * (integrand[:, 1:] + integrand[:, :-1]) * np.diff(e)[None, :], axis=1)
    mean = FINE_STRUCTURE_OVER_HBARC * integral * (step / 10.0)
    counts = rng.poisson(mean)
    bi = 1.0 / beta
    max_cos = bi / nmax
    g[:, 4, 0] = bi
    g[:, 5, 0] = (1.0 - max_cos) * (1.0 + max_cos)
    g[:, 5, 1] = mean
    g[:, 5, 2] = mean
    g[:, 4, 3] = max_cos
    gu[:, 0, 3] = counts
    g[:, 1, 0:3] = pos
    g[:, 1, 3] = 0.0
    g[:, 2, 0:3] = d
    g[:, 2, 3] = step
    g[:, 3, 1] = 1.0                                  # charge
    g[:, 3, 2] = 1.0                                  # weight
    g[:, 3, 3] = beta * G.C_LIGHT                     # preVelocity
    g[:, 5, 3] = beta * G.C_LIGHT                     # postVelocity
    g[:, 4, 1] = float(table[:, 0].min())             # Wmin
    g[:, 4, 2] = float(table[:, 0].max())             # Wmax
    return g


def total_photons(gs):
    return int(gs.view(np.uint32)[:, 0, 3].astype(np.int64).sum())


def seed_array(gs):
    counts = gs.view(np.uint32)[:, 0, 3].astype(np.int64)
    return np.repeat(np.arange(len(gs), dtype=np.int32), counts)
