"""ctypes binding of the CPU oracle (liboracle.so) and of the reference-header build (_ref/libref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` as the checker and by bench.py's
CPU-baseline leg.  Nothing on the product path imports this module.
"""
import ctypes as C
import os
import subprocess
import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REFLIB = os.path.join(HERE, "_ref", "libref.so")
REFDEV_CUBIN = os.path.join(HERE, "_ref", "ref_device.cubin")
REFDEV_RUN = os.path.join(HERE, "_ref", "libref_device_run.so")


class Tex(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("ncomp", C.c_int), ("data", C.c_void_p)]


class Geom(C.Structure):
    _fields_ = [("node", C.c_void_p), ("prim", C.c_void_p), ("solid", C.c_void_p), ("num_solid", C.c_int),
                ("inst", C.c_void_p), ("inst_inv", C.c_void_p), ("num_inst", C.c_int),
                ("itra", C.c_void_p), ("plan", C.c_void_p)]


class Sim(C.Structure):
    _fields_ = [("geom", Geom), ("bnd", Tex), ("bnd_nm0", C.c_float), ("bnd_nms", C.c_float),
                ("optical", C.c_void_p), ("icdf", Tex), ("hd_factor", C.c_int), ("max_bounce", C.c_int),
                ("max_time", C.c_float), ("tmin", C.c_float), ("tmin0", C.c_float), ("tmax", C.c_float),
                ("eps0_mask", C.c_uint32), ("seed", C.c_uint64), ("offset", C.c_uint64),
                ("skipahead_event_offset", C.c_uint64), ("debug_tag", C.c_int)]


def build(ref=False):
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])
    if ref:
        subprocess.check_call(["make", "-s", "-C", HERE, "ref"])


def _ptr(a):
    return a.ctypes.data_as(C.c_void_p)


# flags after which the smaller epsilon applies: TO,CK,SI,SC,RE (sysrap/SEventConfig.cc:104)
EPS0_MASK = (1 << 2) | (1 << 0) | (1 << 1) | (1 << 5) | (1 << 4)


class SimConfig:
    """Owns the arrays a Sim struct points at (so they outlive the ctypes struct)."""

    def __init__(self, arrays, max_bounce=31, max_time=1e27, tmin=0.05, tmin0=0.05, tmax=1e6, seed=0, offset=0,
                 skipahead=100000, debug_tag=1):
        from_geom = arrays
        self.node = np.ascontiguousarray(from_geom["node"], dtype=np.float32)
        self.prim = np.ascontiguousarray(from_geom["prim"], dtype=np.float32)
        self.solid = np.ascontiguousarray(from_geom["solid"])
        self.inst = np.ascontiguousarray(from_geom["inst"], dtype=np.float32)
        self.inst_inv = np.ascontiguousarray(invert_instances(self.inst))
        self.itra = np.ascontiguousarray(from_geom["itra"], dtype=np.float32)
        if self.itra.size == 0:
            self.itra = np.zeros((1, 4, 4), dtype=np.float32)
        self.plan = np.ascontiguousarray(from_geom["plan"], dtype=np.float32)
        if self.plan.size == 0:
            self.plan = np.zeros((1, 4), dtype=np.float32)
        bnd = np.ascontiguousarray(from_geom["bnd"], dtype=np.float32)
        self.bnd_tex = bnd.reshape(-1, bnd.shape[-2], 4)          # (num_bnd*4*2, 761, 4)
        self.optical = np.ascontiguousarray(from_geom["optical"], dtype=np.uint32)
        self.icdf = np.ascontiguousarray(from_geom["icdf"], dtype=np.float32)
        nm0, nms = from_geom["domain"]
        s = Sim()
        s.geom = Geom(_ptr(self.node), _ptr(self.prim), _ptr(self.solid), len(self.solid), _ptr(self.inst),
                      _ptr(self.inst_inv), len(self.inst), _ptr(self.itra), _ptr(self.plan))
        s.bnd = Tex(self.bnd_tex.shape[1], self.bnd_tex.shape[0], 4, _ptr(self.bnd_tex))
        s.bnd_nm0 = nm0
        s.bnd_nms = nms
        s.optical = _ptr(self.optical)
        s.icdf = Tex(self.icdf.shape[1], self.icdf.shape[0], 1, _ptr(self.icdf))
        s.hd_factor = int(from_geom["hd_factor"])
        s.max_bounce = max_bounce
        s.max_time = max_time
        s.tmin = tmin
        s.tmin0 = tmin0
        s.tmax = tmax
        s.eps0_mask = EPS0_MASK
        s.seed = seed
        s.offset = offset
        s.skipahead_event_offset = skipahead
        s.debug_tag = debug_tag
        self.sim = s


def invert_instances(inst):
    """Inverse instance transforms with the same double-precision adjugate formula the engine uses."""
    inst = np.ascontiguousarray(inst, dtype=np.float32)
    out = np.zeros_like(inst)
    lib().orc_invert_transforms(_ptr(inst), _ptr(out), C.c_int(len(inst)))
    return out


class _Lib:
    def __init__(self, path, prefix):
        self.lib = C.CDLL(path)
        self.prefix = prefix


_oracle = None
_ref = None


def lib():
    global _oracle
    if _oracle is None:
        if not os.path.exists(LIB):
            build()
        _oracle = C.CDLL(LIB)
        _oracle.orc_fill_seed.restype = C.c_int64
        _oracle.orc_select_hits.restype = C.c_int64
        _oracle.orc_intersect_prim_c.restype = C.c_int
        _oracle.orc_merge_hits.restype = C.c_int64
    return _oracle


def reflib():
    global _ref
    if _ref is None:
        if not os.path.exists(REFLIB):
            return None
        _ref = C.CDLL(REFLIB)
        _ref.ref_intersect_prim.restype = C.c_int
    return _ref


def simulate(cfg, gs, input_photon=None, event_index=0, photon_offset=0, nthreads=1, seq=True, use_ref=False):
    """Run the oracle (or the reference-header build) over every photon of ``gs``. Returns (photons, seq)."""
    from importlib import import_module
    L = import_module("eic_opticks_gb300.layout")
    gs = np.ascontiguousarray(gs, dtype=np.float32)
    counts = gs.view(np.uint32)[:, 0, 3].astype(np.int64)
    seed = np.ascontiguousarray(np.repeat(np.arange(len(gs), dtype=np.int32), counts))
    n = len(seed)
    out = np.zeros(n, dtype=L.PHOTON)
    sq = np.zeros(n, dtype=L.SEQ) if seq else None
    inp = np.ascontiguousarray(input_photon) if input_photon is not None else np.zeros(1, dtype=L.PHOTON)
    if use_ref:
        r = reflib()
        if r is None:
            raise RuntimeError("reference build oracle/_ref/libref.so not present")
        r.ref_simulate(C.byref(cfg.sim), _ptr(gs), _ptr(seed), _ptr(inp), C.c_uint64(photon_offset),
                       C.c_uint32(event_index), C.c_int64(n), _ptr(out), _ptr(sq) if sq is not None else None)
    else:
        lib().orc_simulate(C.byref(cfg.sim), _ptr(gs), _ptr(seed), _ptr(inp), C.c_uint64(photon_offset),
                           C.c_uint32(event_index), C.c_int64(n), _ptr(out),
                           _ptr(sq) if sq is not None else None, C.c_int(nthreads))
    return out, sq


_refdev = None


def ref_device_cubin(variant=""):
    return REFDEV_CUBIN if not variant else os.path.join(HERE, "_ref", "ref_device_%s.cubin" % variant)


def ref_device_available(variant=""):
    """True when the reference-header device build (ref_device[_variant].cubin) is present."""
    return os.path.exists(ref_device_cubin(variant))


def ref_device_lib():
    global _refdev
    if _refdev is None:
        if not os.path.exists(REFDEV_RUN):
            subprocess.check_call(["make", "-s", "-C", HERE, "ref-device-run"])
        _refdev = C.CDLL(REFDEV_RUN)
        _refdev.ref_device_simulate.restype = C.c_int
        _refdev.ref_device_last_error.restype = C.c_char_p
    return _refdev


def ref_device_simulate(cfg, gs, input_photon=None, event_index=0, variant=""):
    """Run the reference's own headers, compiled by nvcc for the GPU (ref_device.cu), over every photon of ``gs``
    on the current GPU, one thread per photon.  variant "nofma": the build without multiply-add contraction.
    Returns (photons, seq, kernel_ms)."""
    from importlib import import_module
    L = import_module("eic_opticks_gb300.layout")
    cubin = ref_device_cubin(variant)
    if not os.path.exists(cubin):
        raise RuntimeError("reference device build %s not present" % cubin)
    gs = np.ascontiguousarray(gs, dtype=np.float32)
    counts = gs.view(np.uint32)[:, 0, 3].astype(np.int64)
    seed = np.ascontiguousarray(np.repeat(np.arange(len(gs), dtype=np.int32), counts))
    n = len(seed)
    if input_photon is not None:
        input_photon = np.ascontiguousarray(input_photon)
        if len(input_photon) < n:
            raise ValueError("%d input photons for %d photons" % (len(input_photon), n))
    out = np.zeros(n, dtype=L.PHOTON)
    sq = np.zeros(n, dtype=L.SEQ)
    sizes = np.array([len(cfg.node), len(cfg.prim), len(cfg.solid), len(cfg.itra), len(cfg.plan), len(cfg.optical)],
                     dtype=np.int32)
    ms = C.c_float(0.0)
    lib_ = ref_device_lib()
    rc = lib_.ref_device_simulate(cubin.encode(), C.byref(cfg.sim), _ptr(sizes), _ptr(gs), C.c_int64(len(gs)),
                                  _ptr(seed), _ptr(input_photon) if input_photon is not None else None,
                                  C.c_uint64(0), C.c_int32(event_index), C.c_int64(n), _ptr(out), _ptr(sq),
                                  C.byref(ms))
    if rc != 0:
        raise RuntimeError("reference device build: " + lib_.ref_device_last_error().decode())
    return out, sq, ms.value


def trace(cfg, pos, dirs, tmin=0.05, tmax=1e9):
    """Closest hit of each ray by the binary32 brute-force oracle (orc_csg.c): (t, boundary), t = -1 on a miss."""
    pos = np.ascontiguousarray(pos, dtype=np.float32).reshape(-1, 3)
    dirs = np.ascontiguousarray(dirs, dtype=np.float32).reshape(-1, 3)
    t = np.full(len(pos), -1.0, dtype=np.float32)
    b = np.full(len(pos), 0xffffffff, dtype=np.uint32)
    prd = np.zeros(8, dtype=np.float32)
    for i in range(len(pos)):
        lib().orc_trace_c(C.byref(cfg.sim.geom), _ptr(pos[i]), _ptr(dirs[i]), C.c_float(tmin), C.c_float(tmax),
                          _ptr(prd))
        bnd = int(prd.view(np.uint32)[7]) & 0xffff
        if bnd != 0xffff:
            t[i] = prd[3]
            b[i] = bnd
    return t, b


def trace64(cfg, pos, dirs, tmin=0.05, tmax=1e9, nthreads=None):
    """Closest-hit distances in binary64 (orc_csg64.c) for rays given as float32 (n,3) arrays; -1 on a miss."""
    import os as _os
    pos = np.ascontiguousarray(pos, dtype=np.float32)
    dirs = np.ascontiguousarray(dirs, dtype=np.float32)
    n = len(pos)
    t = np.zeros(n, dtype=np.float64)
    b = np.zeros(n, dtype=np.uint32)
    lib().orc_trace64_batch(C.byref(cfg.sim.geom), _ptr(pos), _ptr(dirs), C.c_int64(n), C.c_double(tmin),
                            C.c_double(tmax), _ptr(t), _ptr(b), C.c_int(nthreads or _os.cpu_count() or 1))
    return t, b


def merge_hits(hits, time_window):
    """Hits merged by (identity, time bucket) as the reference's SPM::merge_partial_select does (orc_qsim.c)."""
    hits = np.ascontiguousarray(hits)
    out = np.zeros_like(hits)
    m = lib().orc_merge_hits(_ptr(hits), C.c_int64(len(hits)), C.c_float(time_window), _ptr(out))
    return out[:m]


def philox_uniforms(seed, subsequence, offset, skip, n, use_ref=False):
    out = np.zeros(n, dtype=np.float32)
    if use_ref:
        reflib().ref_curand_uniforms(C.c_uint64(seed), C.c_uint64(subsequence), C.c_uint64(offset),
                                     C.c_uint64(skip), C.c_int(n), _ptr(out))
    else:
        lib().orc_philox_uniforms(C.c_uint64(seed), C.c_uint64(subsequence), C.c_uint64(offset),
                                  C.c_uint64(skip), C.c_int(n), _ptr(out))
    return out


def intersect_prim(node, plan, itra, t_min, o, d, use_ref=False):
    node = np.ascontiguousarray(node, dtype=np.float32)
    plan = np.ascontiguousarray(plan if plan is not None and len(plan) else np.zeros((1, 4)), dtype=np.float32)
    itra = np.ascontiguousarray(itra if itra is not None and len(itra) else np.zeros((1, 4, 4)), dtype=np.float32)
    o = np.ascontiguousarray(o, dtype=np.float32)
    d = np.ascontiguousarray(d, dtype=np.float32)
    out = np.zeros(4, dtype=np.float32)
    if use_ref:
        v = reflib().ref_intersect_prim(_ptr(node), _ptr(plan), _ptr(itra), C.c_float(t_min), _ptr(o), _ptr(d), _ptr(out))
    else:
        v = lib().orc_intersect_prim_c(_ptr(node), _ptr(plan), _ptr(itra), C.c_float(t_min), _ptr(o), _ptr(d), _ptr(out))
    return bool(v), out


def tex_lookup(tex, xy):
    """CUDA linear-filter emulation: tex is (ny, nx) float or (ny, nx, 4) float4; xy (n, 2) normalized coords."""
    tex = np.ascontiguousarray(tex, dtype=np.float32)
    xy = np.ascontiguousarray(xy, dtype=np.float32)
    n = len(xy)
    if tex.ndim == 3:
        t = Tex(tex.shape[1], tex.shape[0], 4, _ptr(tex))
        out = np.zeros((n, 4), dtype=np.float32)
        lib().orc_tex_lookup4(C.byref(t), _ptr(xy), C.c_int(n), _ptr(out))
    else:
        t = Tex(tex.shape[1], tex.shape[0], 1, _ptr(tex))
        out = np.zeros(n, dtype=np.float32)
        lib().orc_tex_lookup1(C.byref(t), _ptr(xy), C.c_int(n), _ptr(out))
    return out
