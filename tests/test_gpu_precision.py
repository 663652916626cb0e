"""Intersection distances of the engine against the binary64 oracle on the large instanced geometry.

Geometry: 17.7 m acrylic sphere of liquid scintillator, 20,000 instanced sensors (depth-3 CSG union of an
ellipsoid and two cylinders, plus the cap prim) on a 19.4 m Fibonacci sphere.  1M rays: half start uniformly inside
r < 17 m with isotropic directions (the acrylic sphere roots, t up to 35 m), half start in the water between the
acrylic and the sensors and aim at the sensors in front of them (the CSG sensor roots).  The engine's distances (binary32, with
and without its binary64 root polish) are compared with orc_csg64.c for the rays whose closest boundary agrees.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rays(n, seed=5):
    rng = np.random.default_rng(seed)
    h = n // 2
    u = rng.normal(size=(n, 3))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = np.concatenate([17000.0 * rng.uniform(0, 1, h) ** (1.0 / 3.0), rng.uniform(17900.0, 18900.0, n - h)])
    pos = r[:, None] * u
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    aim = 19400.0 * u[h:] + rng.normal(scale=300.0, size=(n - h, 3))     # the sensors in front of the start
    a = aim - pos[h:]
    d[h:] = a / np.linalg.norm(a, axis=1, keepdims=True)
    return pos.astype(np.float32), d.astype(np.float32)


def test_fp64_intersection_error_large_geometry(oracle):
    import __graft_entry__ as ge
    ge.build()
    from eic_opticks_gb300 import engine as E, geometry as G
    arrays = G.large_sphere().arrays()
    pos, d = rays(1_000_000)
    t64, b64 = oracle.trace64(oracle.SimConfig(arrays), pos, d)
    h = len(pos) // 2
    out = {}
    for precision in (0, 1):
        eng = E.Engine(arrays, precision=precision)
        t, b = eng.trace_rays(pos, d)
        eng.close()
        for part, sl in (("inside", slice(0, h)), ("sensors", slice(h, None))):
            ok = (b[sl] == b64[sl]) & (t64[sl] > 0) & (t[sl] > 0)
            err = np.abs(t[sl][ok].astype(np.float64) - t64[sl][ok])
            ulp = np.spacing(t64[sl][ok].astype(np.float32)).astype(np.float64)
            q = np.percentile(err, [50, 99, 99.9, 99.99])
            out[precision, part] = (ok.mean(), err.max(), q[2], (err / ulp).max())
            print("precision %d %-7s: same boundary %.6f, |dt| mm p50 %.3g p99 %.3g p99.9 %.3g p99.99 %.3g max %.3g;"
                  " > 1e-3 mm %.2e; max %.1f ulp(t)" % (precision, part, ok.mean(), q[0], q[1], q[2], q[3], err.max(),
                                                         (err > 1e-3).mean(), (err / ulp).max()))
    for part in ("inside", "sensors"):
        assert out[0, part][0] > 0.999 and out[1, part][0] > 0.999
        assert out[1, part][1] <= out[0, part][1] and out[1, part][2] <= out[0, part][2]
    assert out[1, "inside"][3] <= 1.0          # polished sphere roots: within one binary32 ulp of t


@pytest.mark.parametrize("name", ["nested_boxes", "crystal_array", "water_cube"])
def test_fp64_intersection_error_other_geometries(oracle, name):
    """1M rays from points uniform in the inner 95% of the world box, isotropic directions; same report and
    bounds as above (box faces are single-division roots, so both modes sit within a few ulp of t)."""
    import __graft_entry__ as ge
    ge.build()
    from eic_opticks_gb300 import engine as E, geometry as G
    arrays = getattr(G, name)().arrays()
    half = np.abs(arrays["prim"].view(np.float32)[0, 2, :3]).min() * 0.95
    rng = np.random.default_rng(11)
    n = 1_000_000
    pos = rng.uniform(-half, half, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    t64, b64 = oracle.trace64(oracle.SimConfig(arrays), pos, d)
    out = {}
    for precision in (0, 1):
        eng = E.Engine(arrays, precision=precision)
        t, b = eng.trace_rays(pos, d)
        eng.close()
        ok = (b == b64) & (t64 > 0) & (t > 0)
        err = np.abs(t[ok].astype(np.float64) - t64[ok])
        ulp = np.spacing(t64[ok].astype(np.float32)).astype(np.float64)
        q = np.percentile(err, [50, 99, 99.9])
        out[precision] = (ok.mean(), err.max(), (err / ulp).max())
        print("%s precision %d: same boundary %.6f, |dt| mm p50 %.3g p99 %.3g p99.9 %.3g max %.3g; max %.1f ulp(t)"
              % (name, precision, ok.mean(), q[0], q[1], q[2], err.max(), (err / ulp).max()))
    assert out[0][0] > 0.999 and out[1][0] > 0.999
    assert out[1][1] <= out[0][1] * 1.0001 + 1e-9


@pytest.mark.parametrize("fixture", ["sim_crystal_array.npz", "sim_large_sphere_small.npz"])
def test_precision_mode_kernel_forms_agree(fixture):
    """The precision mode in every kernel form (one thread per photon, photon pool over pregenerated photons,
    wavefront carrying each photon's binary64 accumulators between its passes): the same flag histories, flags,
    indices and hits; float words within the kernel-form bounds, or, on the mirrored small sphere whose paths grow
    last-bit differences between separately compiled kernels, within 1e-3 mm / 1e-3 ns for at least as many photons
    as the reference's own builds agree on."""
    import __graft_entry__ as ge
    ge.build()
    from conftest import assert_forms_agree, golden_arrays, load_golden
    from eic_opticks_gb300 import engine as E
    z = load_golden(fixture)
    arrays = golden_arrays(z)
    out = {}
    for mode in (1, 2, 3):
        eng = E.Engine(arrays, precision=1, record_photon=1, record_seq=1, kernel_mode=mode)
        eng.simulate(int(z["event_index"]), z["gs"])
        out[mode] = (eng.photons(), eng.seq(), eng.hits())
        eng.close()
    for mode in (2, 3):
        assert np.array_equal(out[mode][1].view(np.uint64), out[1][1].view(np.uint64))
        assert np.array_equal(out[mode][2]["index"], out[1][2]["index"])
        assert_forms_agree(out[mode][0], out[1][0], fixture)
