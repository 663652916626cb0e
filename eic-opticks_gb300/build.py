"""Compile recipe for libgbopticks.so (sm_103a) : explicit nvcc / g++ invocations, no cmake.

The library is built in-tree at ``eic-opticks_gb300/libgbopticks.so`` so that a process loading it shows the
in-tree path.  Host C++ is compiled with -ffp-contract=off so that the inverse instance transforms are the same
binary32 values on x86-64 and aarch64 hosts.

``build(variant="nofma")`` compiles the same sources with nvcc's --fmad=false into
``eic-opticks_gb300/libgbopticks_nofma.so``: every binary32 multiply and add rounded on its own, so that results
depend only on the order of operations written in the source.  The parity tests use it to check the engine's
arithmetic operation for operation against the reference's headers compiled the same way; it is not a product
build (contraction stays on there, as in the reference's own build).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbopticks.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["gbo_engine.cu", "gbo_sim_tree0.cu", "gbo_sim_tree1.cu", "gbo_sim_tree2.cu", "gbo_merge.cu"]
CPP_SOURCES = ["gbo_accel.cpp"]
HEADERS = ["gbo_device.cuh", "gbo_csg.cuh", "gbo_physics.cuh", "gbo_trace.cuh", "gbo_accel.h", "gbo_serve.inl",
           "gbo_merge.h", "gbo_sim.cuh", "gbo_sim_forms.inl"]


def _newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


VARIANTS = {"": [], "nofma": ["--fmad=false"]}


def library_path(variant=""):
    return LIB if not variant else os.path.join(HERE, "libgbopticks_%s.so" % variant)


def build(verbose=False, force=False, ptxas_verbose=False, variant=""):
    lib_path = library_path(variant)
    build_dir = BUILD if not variant else os.path.join(BUILD, variant)
    os.makedirs(build_dir, exist_ok=True)
    inc = os.path.join(os.path.dirname(HERE), "include")
    deps = [os.path.join(CSRC, f) for f in CU_SOURCES + CPP_SOURCES + HEADERS]
    deps += [os.path.join(inc, f) for f in ("gbopticks.h", "gbo_types.h")]
    if not force and not _newer(lib_path, deps):
        return lib_path
    procs, objs = [], []
    for f in CU_SOURCES:
        o = os.path.join(build_dir, f + ".o")
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", inc, *VARIANTS[variant],
               "-c", os.path.join(CSRC, f), "-o", o]
        extra = os.environ.get("GBO_NVCC_DEFINES", "").split()      # tuning builds: -DGBO_SIM_MINB=5, --fmad=false
        cmd[1:1] = [x for x in extra if x.startswith("-D") or x.startswith("--fmad=")]
        if ptxas_verbose:
            cmd[1:1] = ["-Xptxas", "-v"]
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
        objs.append(o)
    for f in CPP_SOURCES:
        o = os.path.join(build_dir, f + ".o")
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", inc, "-c", os.path.join(CSRC, f), "-o", o]
        procs.append(subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT))
        objs.append(o)
    logs = []
    for p in procs:
        out, _ = p.communicate()
        logs.append(out.decode(errors="replace"))
        if p.returncode != 0:
            sys.stderr.write(out.decode(errors="replace"))
            raise RuntimeError("compile failed: %s" % " ".join(p.args))
    tmp = lib_path + ".tmp"
    link = [NVCC, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    subprocess.check_call(link)
    os.replace(tmp, lib_path)
    if verbose or ptxas_verbose:
        for lg in logs:
            if lg.strip():
                print(lg)
    return lib_path


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv, ptxas_verbose="-v" in sys.argv)
