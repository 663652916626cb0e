"""The C-ABI library loads without a GPU and exports every entry point include/*.h declares."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in os.listdir(os.path.join(ROOT, "include")):
        if not h.endswith(".h"):
            continue
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(gbo_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as ge
    ge.load_package()
    from eic_opticks_gb300 import build
    path = build.build()
    return ctypes.CDLL(path)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for must in ("gbo_engine_create", "gbo_simulate", "gbo_num_hit", "gbo_copy_hits", "gbo_reset"):
        assert must in syms


def test_library_exports_declared_symbols(lib):
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_config_default_without_gpu(lib, monkeypatch):
    from eic_opticks_gb300 import engine as E
    monkeypatch.setenv("OPTICKS_MAX_BOUNCE", "9")
    monkeypatch.setenv("OPTICKS_HIT_MASK", "SD,EC")
    c = E.Config()
    assert lib.gbo_config_default(ctypes.byref(c)) == 0
    assert c.max_bounce == 9
    assert c.hit_mask == (1 << 6) | (1 << 13)
    assert abs(c.propagate_epsilon - 0.05) < 1e-9 and c.event_skipahead == 100000 and c.debug_tag == 1


def test_engine_create_rejects_bad_geometry(lib):
    from eic_opticks_gb300 import engine as E
    d = E.GeometryDesc()
    h = ctypes.c_void_p()
    lib.gbo_last_error.restype = ctypes.c_char_p
    rc = lib.gbo_engine_create(ctypes.byref(d), None, 0, ctypes.byref(h))
    assert rc == 1 and b"missing" in lib.gbo_last_error()


def test_event_api_argument_errors_without_gpu(lib):
    """The engine-handle event API refuses a null engine before touching the GPU."""
    lib.gbo_event_num_hits.restype = ctypes.c_int64
    t = ctypes.c_uint64()
    assert lib.gbo_event_submit(None, None, ctypes.c_size_t(0), ctypes.c_uint32(1), ctypes.byref(t)) == 1
    assert lib.gbo_event_wait(None, ctypes.c_uint64(1), ctypes.c_int64(0)) == 1
    assert lib.gbo_event_num_hits(None, ctypes.c_uint64(1)) < 0
    assert lib.gbo_event_copy_hits(None, ctypes.c_uint64(1), None, ctypes.c_size_t(0)) == 1
    assert lib.gbo_event_release(None, ctypes.c_uint64(1)) == 1


def test_ctypes_mirrors_match_the_header(tmp_path):
    """Every ctypes structure of the Python binding has the size and field offsets the C compiler gives the header's
    struct (a field added on one side only would shift every later field)."""
    import subprocess
    from eic_opticks_gb300 import engine as E
    pairs = [("gbo_config", E.Config), ("gbo_tune_result", E.TuneResult), ("gbo_stats", E.Stats),
             ("gbo_geometry_desc", E.GeometryDesc), ("gbo_server_config", E.ServerConfig),
             ("gbo_server_stats", E.ServerStats)]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbopticks.h"', "int main(void) {"]
    for cname, py in pairs:
        lines.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines.append("return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines))
    exe = tmp_path / "layout"
    subprocess.check_call(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    got = dict(l.split() for l in subprocess.check_output([str(exe)]).decode().split("\n") if l)
    for cname, py in pairs:
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got["%s.%s" % (cname, f)]) == getattr(py, f).offset, (cname, f)
