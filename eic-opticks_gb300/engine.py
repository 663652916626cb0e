"""ctypes binding of libgbopticks.so and a ``G4CXOpticks``-shaped facade over it.

The facade keeps the reference's call sequence (g4cx/G4CXOpticks.hh:38-107, sysrap/SEvt.hh:487, SEvt.cc:2050,4991):

    gx = G4CXOpticks.SetGeometry(geometry_arrays)      # once
    SEvt.AddGenstep(quad6) ... / SEvt.SetInputPhoton(photons)
    gx.simulate(eventID, reset=False)                   # synchronous
    n = SEvt.GetNumHit(0); hits = SEvt.GetHits()
    gx.reset(eventID)

Errors from the library raise ``GBOError`` carrying the library's message.  There is no fallback: if the CUDA
library is missing or no GPU is present, construction fails loudly.
"""
import ctypes as C
import os

import numpy as np

from . import gensteps as GS
from . import layout as L

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libgbopticks.so")


class GBOError(RuntimeError):
    pass


class GeometryDesc(C.Structure):
    _fields_ = [("node", C.c_void_p), ("num_node", C.c_int32), ("prim", C.c_void_p), ("num_prim", C.c_int32),
                ("solid", C.c_void_p), ("num_solid", C.c_int32), ("inst", C.c_void_p), ("num_inst", C.c_int32),
                ("itra", C.c_void_p), ("num_itra", C.c_int32), ("plan", C.c_void_p), ("num_plan", C.c_int32),
                ("bnd", C.c_void_p), ("num_bnd", C.c_int32), ("bnd_nx", C.c_int32),
                ("bnd_domain_low", C.c_float), ("bnd_domain_step", C.c_float), ("optical", C.c_void_p),
                ("icdf", C.c_void_p), ("icdf_ny", C.c_int32), ("icdf_nx", C.c_int32), ("hd_factor", C.c_int32)]


class Config(C.Structure):
    _fields_ = [("max_bounce", C.c_int32), ("max_time", C.c_float), ("propagate_epsilon", C.c_float),
                ("propagate_epsilon0", C.c_float), ("epsilon0_mask", C.c_uint32), ("hit_mask", C.c_uint32),
                ("rng_seed", C.c_uint64), ("rng_offset", C.c_uint64), ("event_skipahead", C.c_uint64),
                ("tmax", C.c_float), ("debug_tag", C.c_int32), ("record_photon", C.c_int32),
                ("record_seq", C.c_int32), ("max_photon", C.c_int64), ("kernel_mode", C.c_int32),
                ("refill_min", C.c_int32), ("blocks_per_sm", C.c_int32), ("refill_period", C.c_int32),
                ("max_slot", C.c_int64), ("precision", C.c_int32), ("walk_min", C.c_int32),
                ("rng_call", C.c_int32), ("reserved", C.c_int32)]


class TuneResult(C.Structure):
    _fields_ = [("kernel_mode", C.c_int32), ("refill_min", C.c_int32), ("refill_period", C.c_int32),
                ("num_candidates", C.c_int32), ("cand_mode", C.c_int32 * 32), ("cand_refill", C.c_int32 * 32),
                ("cand_period", C.c_int32 * 32), ("cand_ms", C.c_float * 32), ("blocks_per_sm", C.c_int32),
                ("cand_blocks", C.c_int32 * 32), ("walk_min", C.c_int32), ("cand_walk", C.c_int32 * 32),
                ("rng_call", C.c_int32), ("cand_rng_call", C.c_int32 * 32)]


class Stats(C.Structure):
    _fields_ = [("num_photon", C.c_int64), ("num_hit", C.c_int64), ("ms_upload", C.c_float),
                ("ms_simulate", C.c_float), ("ms_compact", C.c_float), ("simulate_launches", C.c_int32),
                ("kernel_launches", C.c_int32), ("ms_generate", C.c_float), ("reserved", C.c_int32)]


EXPORTS = ["gbo_config_default", "gbo_engine_create", "gbo_engine_destroy", "gbo_simulate", "gbo_simulate_device",
           "gbo_num_hit", "gbo_num_photon", "gbo_copy_hits", "gbo_copy_photons", "gbo_copy_seq", "gbo_device_hits",
           "gbo_reset", "gbo_get_stats", "gbo_last_error"]

_lib = None


def load(path=None):
    """Load the library (built by ``eic_opticks_gb300.build``); raises if it is missing.  GBO_ENGINE_LIBRARY may
    name another build of the same sources (the parity tests' --fmad=false build)."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or os.environ.get("GBO_ENGINE_LIBRARY") or LIB
    if not os.path.exists(path):
        raise GBOError("libgbopticks.so not built (%s): run __graft_entry__.build()" % path)
    lib = C.CDLL(path)
    lib.gbo_last_error.restype = C.c_char_p
    lib.gbo_num_hit.restype = C.c_int64
    lib.gbo_num_photon.restype = C.c_int64
    lib.gbo_device_hits.restype = C.c_void_p
    lib.gbo_engine_create.argtypes = [C.POINTER(GeometryDesc), C.POINTER(Config), C.c_int, C.POINTER(C.c_void_p)]
    lib.gbo_engine_destroy.argtypes = [C.c_void_p]
    lib.gbo_simulate.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64]
    lib.gbo_simulate_device.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p]
    lib.gbo_simulate_slice.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_uint64]
    lib.gbo_simulate_to_host.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_void_p,
                                         C.c_int64, C.POINTER(C.c_int64)]
    lib.gbo_num_hit.argtypes = [C.c_void_p]
    lib.gbo_num_photon.argtypes = [C.c_void_p]
    lib.gbo_device_hits.argtypes = [C.c_void_p]
    for f in ("gbo_copy_hits", "gbo_copy_photons", "gbo_copy_seq", "gbo_copy_merged_hits"):
        getattr(lib, f).argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_int64]
    lib.gbo_merge_hits.argtypes = [C.c_void_p, C.c_float, C.POINTER(C.c_int64)]
    lib.gbo_merge_hits_device.argtypes = [C.c_void_p, C.c_int64, C.c_float, C.c_void_p, C.POINTER(C.c_int64),
                                          C.c_void_p]
    lib.gbo_reset.argtypes = [C.c_void_p, C.c_int32]
    lib.gbo_get_stats.argtypes = [C.c_void_p, C.POINTER(Stats)]
    lib.gbo_rng_sequence.argtypes = [C.c_int, C.c_uint64, C.c_uint64, C.c_uint64, C.c_int32, C.c_int32, C.c_void_p]
    lib.gbo_texture_lookup.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p]
    lib.gbo_scint_wavelength.argtypes = [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]
    lib.gbo_trace_rays.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_float, C.c_float, C.c_void_p,
                                   C.c_void_p]
    lib.gbo_autotune.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32,
                                 C.c_void_p]
    _lib = lib
    return lib


def rng_sequence(seed, subsequence0, position, num_seq, per_seq, device=0):
    lib = load()
    out = np.zeros((num_seq, per_seq), dtype=np.float32)
    _check(lib.gbo_rng_sequence(device, seed, subsequence0, position, num_seq, per_seq,
                                out.ctypes.data_as(C.c_void_p)), "gbo_rng_sequence")
    return out


def _check(rc, what):
    if rc != 0:
        raise GBOError("%s failed (code %d): %s" % (what, rc, _lib.gbo_last_error().decode()))


def default_config(**kw):
    lib = load()
    c = Config()
    _check(lib.gbo_config_default(C.byref(c)), "gbo_config_default")
    for k, v in kw.items():
        setattr(c, k, v)
    return c


class Engine:
    """One GPU engine holding geometry, tables and event buffers (thin wrapper over the C ABI)."""

    def __init__(self, arrays, config=None, device=0, **config_kw):
        lib = load()
        self._keep = {k: np.ascontiguousarray(arrays[k]) for k in ("node", "prim", "solid", "inst", "itra", "plan",
                                                                     "bnd", "optical", "icdf")}
        a = self._keep
        d = GeometryDesc()
        p = lambda x: x.ctypes.data_as(C.c_void_p)  # noqa: E731
        d.node, d.num_node = p(a["node"]), len(a["node"])
        d.prim, d.num_prim = p(a["prim"]), len(a["prim"])
        d.solid, d.num_solid = p(a["solid"]), len(a["solid"])
        d.inst, d.num_inst = p(a["inst"]), len(a["inst"])
        d.itra, d.num_itra = (p(a["itra"]) if a["itra"].size else None), len(a["itra"])
        d.plan, d.num_plan = (p(a["plan"]) if a["plan"].size else None), len(a["plan"])
        d.bnd, d.num_bnd, d.bnd_nx = p(a["bnd"]), a["bnd"].shape[0], a["bnd"].shape[3]
        d.bnd_domain_low, d.bnd_domain_step = arrays["domain"]
        d.optical = p(a["optical"])
        d.icdf, d.icdf_ny, d.icdf_nx = p(a["icdf"]), a["icdf"].shape[0], a["icdf"].shape[1]
        d.hd_factor = int(arrays["hd_factor"])
        self.config = config if config is not None else default_config(**config_kw)
        h = C.c_void_p()
        _check(lib.gbo_engine_create(C.byref(d), C.byref(self.config), device, C.byref(h)), "gbo_engine_create")
        self.handle = h
        self.lib = lib

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gbo_engine_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def simulate(self, event_id, gensteps, input_photon=None):
        gs = np.ascontiguousarray(gensteps, dtype=np.float32)
        inp = np.ascontiguousarray(input_photon) if input_photon is not None else None
        _check(self.lib.gbo_simulate(self.handle, int(event_id), gs.ctypes.data_as(C.c_void_p), len(gs),
                                     inp.ctypes.data_as(C.c_void_p) if inp is not None else None,
                                     len(inp) if inp is not None else 0), "gbo_simulate")
        return self.num_hit()

    def simulate_to_host(self, event_id, gensteps, out, input_photon=None):
        """gbo_simulate_to_host: simulate and write the hits into `out` (a PHOTON array, page-locked for overlap);
        returns the hit count.  A count above len(out) raises after the first len(out) hits were stored."""
        gs = np.ascontiguousarray(gensteps, dtype=np.float32)
        inp = np.ascontiguousarray(input_photon) if input_photon is not None else None
        if out.dtype != L.PHOTON or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a C-contiguous photon array")
        n = C.c_int64()
        _check(self.lib.gbo_simulate_to_host(self.handle, int(event_id), gs.ctypes.data_as(C.c_void_p), len(gs),
                                             inp.ctypes.data_as(C.c_void_p) if inp is not None else None,
                                             len(inp) if inp is not None else 0, out.ctypes.data_as(C.c_void_p),
                                             len(out), C.byref(n)), "gbo_simulate_to_host")
        return int(n.value)

    def simulate_slice(self, event_id, gensteps, photon_offset, input_photon=None):
        """One launch of the event photons photon_offset.. (gbo_simulate_slice)."""
        gs = np.ascontiguousarray(gensteps, dtype=np.float32)
        inp = np.ascontiguousarray(input_photon) if input_photon is not None else None
        _check(self.lib.gbo_simulate_slice(self.handle, int(event_id), gs.ctypes.data_as(C.c_void_p), len(gs),
                                           inp.ctypes.data_as(C.c_void_p) if inp is not None else None,
                                           len(inp) if inp is not None else 0, C.c_uint64(int(photon_offset))),
               "gbo_simulate_slice")
        return self.num_hit()

    def simulate_device(self, event_id, d_gs_ptr, num_gs, d_input_ptr=0, num_input=0, stream=0):
        _check(self.lib.gbo_simulate_device(self.handle, int(event_id), C.c_void_p(d_gs_ptr), int(num_gs),
                                            C.c_void_p(d_input_ptr) if d_input_ptr else None, int(num_input),
                                            C.c_void_p(stream) if stream else None), "gbo_simulate_device")
        return self.num_hit()

    def num_hit(self):
        return int(self.lib.gbo_num_hit(self.handle))

    def num_photon(self):
        return int(self.lib.gbo_num_photon(self.handle))

    def hits(self, out=None):
        n = self.num_hit()
        if n < 0:       # no event yet: let the library report the state error
            _check(self.lib.gbo_copy_hits(self.handle, None, 0, 0), "gbo_copy_hits")
        out = np.zeros(n, dtype=L.PHOTON) if out is None else out
        _check(self.lib.gbo_copy_hits(self.handle, out.ctypes.data_as(C.c_void_p), 0, n), "gbo_copy_hits")
        return out

    def merge_hits(self, time_window=1.0):
        """The current event's hits merged by (sensor identity, time bucket of time_window ns): gbo_merge_hits."""
        n = C.c_int64()
        _check(self.lib.gbo_merge_hits(self.handle, C.c_float(time_window), C.byref(n)), "gbo_merge_hits")
        out = np.zeros(n.value, dtype=L.PHOTON)
        _check(self.lib.gbo_copy_merged_hits(self.handle, out.ctypes.data_as(C.c_void_p), 0, n.value),
               "gbo_copy_merged_hits")
        return out

    def photons(self):
        n = self.num_photon()
        out = np.zeros(n, dtype=L.PHOTON)
        _check(self.lib.gbo_copy_photons(self.handle, out.ctypes.data_as(C.c_void_p), 0, n), "gbo_copy_photons")
        return out

    def seq(self):
        n = self.num_photon()
        out = np.zeros(n, dtype=L.SEQ)
        _check(self.lib.gbo_copy_seq(self.handle, out.ctypes.data_as(C.c_void_p), 0, n), "gbo_copy_seq")
        return out

    def reset(self, event_id=0):
        _check(self.lib.gbo_reset(self.handle, int(event_id)), "gbo_reset")

    def stats(self):
        s = Stats()
        _check(self.lib.gbo_get_stats(self.handle, C.byref(s)), "gbo_get_stats")
        return {k: getattr(s, k) for k, _ in Stats._fields_}

    def autotune(self, event_id, gensteps, input_photon=None, trials=2):
        """Time every candidate kernel form on this sample event and keep the fastest (gbo_autotune)."""
        gs = np.ascontiguousarray(gensteps, dtype=np.float32)
        inp = np.ascontiguousarray(input_photon) if input_photon is not None else None
        r = TuneResult()
        _check(self.lib.gbo_autotune(self.handle, int(event_id), gs.ctypes.data_as(C.c_void_p), len(gs),
                                     inp.ctypes.data_as(C.c_void_p) if inp is not None else None,
                                     len(inp) if inp is not None else 0, int(trials), C.byref(r)), "gbo_autotune")
        cands = [dict(mode=r.cand_mode[i], refill=r.cand_refill[i], period=r.cand_period[i],
                      blocks_per_sm=r.cand_blocks[i], walk_min=r.cand_walk[i], rng_call=r.cand_rng_call[i],
                      ms=r.cand_ms[i])
                 for i in range(r.num_candidates)]
        self.config.kernel_mode, self.config.refill_min, self.config.refill_period = r.kernel_mode, r.refill_min, r.refill_period
        self.config.blocks_per_sm, self.config.walk_min, self.config.rng_call = r.blocks_per_sm, r.walk_min, r.rng_call
        return dict(kernel_mode=r.kernel_mode, refill_min=r.refill_min, refill_period=r.refill_period,
                    blocks_per_sm=r.blocks_per_sm, walk_min=r.walk_min, rng_call=r.rng_call, candidates=cands)

    def texture_lookup(self, which, xy):
        xy = np.ascontiguousarray(xy, dtype=np.float32)
        out = np.zeros((len(xy), 4), dtype=np.float32)
        _check(self.lib.gbo_texture_lookup(self.handle, int(which), xy.ctypes.data_as(C.c_void_p), len(xy),
                                           out.ctypes.data_as(C.c_void_p)), "gbo_texture_lookup")
        return out if which == 0 else out[:, 0].copy()

    def trace_rays(self, pos, dir, tmin=0.05, tmax=1e6):
        pos = np.ascontiguousarray(pos, dtype=np.float32)
        dir = np.ascontiguousarray(dir, dtype=np.float32)
        t = np.zeros(len(pos), dtype=np.float32)
        b = np.zeros(len(pos), dtype=np.uint32)
        _check(self.lib.gbo_trace_rays(self.handle, pos.ctypes.data_as(C.c_void_p), dir.ctypes.data_as(C.c_void_p),
                                       len(pos), C.c_float(tmin), C.c_float(tmax), t.ctypes.data_as(C.c_void_p),
                                       b.ctypes.data_as(C.c_void_p)), "gbo_trace_rays")
        return t, b

    def scint_wavelength(self, u):
        u = np.ascontiguousarray(u, dtype=np.float32)
        out = np.zeros(len(u), dtype=np.float32)
        _check(self.lib.gbo_scint_wavelength(self.handle, u.ctypes.data_as(C.c_void_p), len(u),
                                             out.ctypes.data_as(C.c_void_p)), "gbo_scint_wavelength")
        return out


class ServerConfig(C.Structure):
    _fields_ = [("slots", C.c_int32), ("max_batch_events", C.c_int32), ("max_batch_photon", C.c_int64),
                ("hbm_budget_bytes", C.c_int64), ("min_batch_photon", C.c_int64), ("use_graph", C.c_int32),
                ("big_exclusive", C.c_int32), ("target_batch_photon", C.c_int64), ("max_wait_us", C.c_int64)]


class ServerStats(C.Structure):
    _fields_ = [("events_submitted", C.c_int64), ("events_done", C.c_int64), ("batches", C.c_int64),
                ("photons", C.c_int64), ("max_batch_photon", C.c_int64), ("graph_launches", C.c_int64),
                ("graph_instantiations", C.c_int64)]


def _server_protos(lib):
    if getattr(lib, "_server_protos", False):
        return
    lib.gbo_server_config_default.argtypes = [C.POINTER(ServerConfig)]
    lib.gbo_server_create.argtypes = [C.c_void_p, C.POINTER(ServerConfig), C.POINTER(C.c_void_p)]
    lib.gbo_server_submit.argtypes = [C.c_void_p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                                      C.POINTER(C.c_uint64)]
    lib.gbo_server_wait.argtypes = [C.c_void_p, C.c_uint64, C.c_int64]
    lib.gbo_server_event_info.argtypes = [C.c_void_p, C.c_uint64, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                          C.POINTER(C.c_double)]
    lib.gbo_server_copy_hits.argtypes = [C.c_void_p, C.c_uint64, C.c_void_p, C.c_int64, C.c_int64]
    lib.gbo_server_release.argtypes = [C.c_void_p, C.c_uint64]
    lib.gbo_server_get_stats.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
    lib.gbo_server_destroy.argtypes = [C.c_void_p]
    lib._server_protos = True


class Server:
    """Continuous-batching event server over an Engine (gbo_server_*): submit from any thread, wait, fetch hits."""

    def __init__(self, engine, **cfg):
        self.lib = engine.lib
        _server_protos(self.lib)
        c = ServerConfig()
        _check(self.lib.gbo_server_config_default(C.byref(c)), "gbo_server_config_default")
        for k, v in cfg.items():
            setattr(c, k, v)
        h = C.c_void_p()
        _check(self.lib.gbo_server_create(engine.handle, C.byref(c), C.byref(h)), "gbo_server_create")
        self.handle = h
        self.engine = engine

    def submit(self, event_id, gensteps, input_photon=None):
        gs = np.ascontiguousarray(gensteps, dtype=np.float32)
        inp = np.ascontiguousarray(input_photon) if input_photon is not None else None
        t = C.c_uint64()
        _check(self.lib.gbo_server_submit(self.handle, int(event_id), gs.ctypes.data_as(C.c_void_p), len(gs),
                                          inp.ctypes.data_as(C.c_void_p) if inp is not None else None,
                                          len(inp) if inp is not None else 0, C.byref(t)), "gbo_server_submit")
        return t.value

    def wait(self, ticket, timeout_us=-1):
        rc = self.lib.gbo_server_wait(self.handle, C.c_uint64(ticket), int(timeout_us))
        if rc == 6:
            return False
        _check(rc, "gbo_server_wait")
        return True

    def info(self, ticket):
        n, h, lat = C.c_int64(), C.c_int64(), C.c_double()
        _check(self.lib.gbo_server_event_info(self.handle, C.c_uint64(ticket), C.byref(n), C.byref(h), C.byref(lat)),
               "gbo_server_event_info")
        return dict(num_photon=n.value, num_hit=h.value, latency_s=lat.value)

    def hits(self, ticket):
        n = self.info(ticket)["num_hit"]
        out = np.zeros(n, dtype=L.PHOTON)
        _check(self.lib.gbo_server_copy_hits(self.handle, C.c_uint64(ticket), out.ctypes.data_as(C.c_void_p), 0, n),
               "gbo_server_copy_hits")
        return out

    def release(self, ticket):
        _check(self.lib.gbo_server_release(self.handle, C.c_uint64(ticket)), "gbo_server_release")

    def stats(self):
        s = ServerStats()
        _check(self.lib.gbo_server_get_stats(self.handle, C.byref(s)), "gbo_server_get_stats")
        return {k: getattr(s, k) for k, _ in ServerStats._fields_}

    def close(self):
        if getattr(self, "handle", None):
            self.lib.gbo_server_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SEvt:
    """Genstep / input-photon collection and hit download, shaped like sysrap/SEvt's static API."""

    _gensteps = []
    _input_photon = None
    _engine = None

    @classmethod
    def AddGenstep(cls, q6):
        cls._gensteps.append(np.asarray(q6, dtype=np.float32).reshape(-1, 6, 4))

    @classmethod
    def SetInputPhoton(cls, photons):
        cls._input_photon = np.ascontiguousarray(photons)
        cls._gensteps = [GS.input_photon_genstep(len(photons))]

    @classmethod
    def GetNumHit(cls, _eidx=0):
        return cls._engine.num_hit() if cls._engine else 0

    @classmethod
    def GetHits(cls):
        return cls._engine.hits()

    @classmethod
    def getHit(cls, idx):
        return cls._engine.hits()[idx]

    @classmethod
    def _take(cls):
        gs = np.concatenate(cls._gensteps) if cls._gensteps else np.zeros((0, 6, 4), np.float32)
        inp = cls._input_photon
        return gs, inp

    @classmethod
    def Clear(cls):
        cls._gensteps = []
        cls._input_photon = None


class G4CXOpticks:
    """SetGeometry / simulate / reset facade (g4cx/G4CXOpticks.hh:49,95-96)."""

    INSTANCE = None

    def __init__(self, arrays, **config_kw):
        self.engine = Engine(arrays, **config_kw)
        SEvt._engine = self.engine

    @classmethod
    def SetGeometry(cls, arrays, **config_kw):
        cls.INSTANCE = cls(arrays, **config_kw)
        return cls.INSTANCE

    @classmethod
    def Get(cls):
        return cls.INSTANCE

    def simulate(self, eventID, reset=False):
        gs, inp = SEvt._take()
        self.engine.simulate(eventID, gs, inp)
        if reset:
            self.reset(eventID)

    def reset(self, eventID):
        SEvt.Clear()
        self.engine.reset(eventID)
