"""Builds libgbcc_sim.so: libgbcc's host sources (the files under
``sisi4s_gb300/csrc`` without device code) compiled by the host C++ compiler
and linked against the host simulation of its device side (``sim.hpp``).
Test infrastructure only.

    python tests/harness/sim/build_sim.py
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(os.path.dirname(HERE)))
CSRC = os.path.join(ROOT, "sisi4s_gb300", "csrc")
OUT = os.path.join(os.path.dirname(HERE), "_build", "sim")
LIB = os.path.join(OUT, "libgbcc_sim.so")
LD_DIR = os.path.join(OUT, "ld")

#: the library's translation units that hold host code only
HOST_UNITS = ["capi.cu", "ccsd.cu", "ccsd_batch.cu", "ccsd_complex.cu", "ccsd_stored.cu", "contract.cu",
              "serve.cu"]
SIM_UNITS = ["sim_runtime.cpp", "sim_kernels.cpp"]


def cuda_include():
    for d in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if d and os.path.exists(os.path.join(d, "include", "cuda_runtime.h")):
            return os.path.join(d, "include")
    raise RuntimeError("cuda_runtime.h not found")


def _deps():
    hdrs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".hpp", ".h"))]
    hdrs += [os.path.join(HERE, "sim.hpp"), os.path.join(ROOT, "include", "gbcc.h")]
    return hdrs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build():
    os.makedirs(OUT, exist_ok=True)
    flags = ["g++", "-std=c++17", "-O2", "-fPIC", "-pthread", "-Wall",
             "-I", cuda_include(), "-I", CSRC, "-I", HERE]
    hdrs = _deps()
    jobs, objs = [], []
    for f in HOST_UNITS + SIM_UNITS:
        src = os.path.join(CSRC if f in HOST_UNITS else HERE, f)
        obj = os.path.join(OUT, f.rsplit(".", 1)[0] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            lang = ["-x", "c++"] if f.endswith(".cu") else []
            jobs.append(flags + lang + ["-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("sim build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))

    with ThreadPoolExecutor(max_workers=min(len(jobs) or 1, os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    if jobs or _stale(LIB, objs + [os.path.abspath(__file__)]):
        # -Bsymbolic: the library's calls into the stand-in runtime bind to
        # it even in a process that has loaded the real CUDA runtime globally
        run(["g++", "-shared", "-pthread", "-Wl,--no-undefined", "-Wl,-Bsymbolic", "-o", LIB]
            + objs)
    # a directory whose libgbcc.so is the simulation: with it first on
    # LD_LIBRARY_PATH the step runner (which links libgbcc.so with a RUNPATH)
    # runs on the simulation too
    link = os.path.join(LD_DIR, "libgbcc.so")
    os.makedirs(LD_DIR, exist_ok=True)
    if not os.path.islink(link):
        os.symlink(os.path.relpath(LIB, LD_DIR), link)
    return LIB


def build_sanitized():
    """The simulation library built with AddressSanitizer and
    UndefinedBehaviorSanitizer; returns (library, directory whose libgbcc.so
    is that library)."""
    out = os.path.join(OUT, "asan")
    ld = os.path.join(out, "ld")
    os.makedirs(ld, exist_ok=True)
    lib = os.path.join(out, "libgbcc_sim_asan.so")
    flags = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
             "-fno-omit-frame-pointer", "-fPIC", "-pthread",
             "-I", cuda_include(), "-I", CSRC, "-I", HERE]
    srcs = [os.path.join(CSRC, f) for f in HOST_UNITS] + [
        os.path.join(HERE, f) for f in SIM_UNITS]
    if _stale(lib, srcs + _deps() + [os.path.abspath(__file__)]):
        def one(src):
            obj = os.path.join(out, os.path.basename(src).rsplit(".", 1)[0] + ".o")
            lang = ["-x", "c++"] if src.endswith(".cu") else []
            r = subprocess.run(flags + lang + ["-c", src, "-o", obj], capture_output=True,
                               text=True)
            if r.returncode != 0:
                raise RuntimeError("sanitized build failed:\n%s" % r.stderr)
            return obj

        with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
            objs = list(ex.map(one, srcs))
        r = subprocess.run(["g++", "-shared", "-fsanitize=address,undefined", "-pthread",
                            "-Wl,-Bsymbolic",
                            "-o", lib] + objs, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("sanitized link failed:\n%s" % r.stderr)
    link = os.path.join(ld, "libgbcc.so")
    if not os.path.islink(link):
        os.symlink(os.path.relpath(lib, ld), link)
    return lib, ld


def build_serve_race():
    """serve_race.cpp linked against a ThreadSanitizer build of the library's
    host code and of the simulation; returns the binary's path."""
    out = os.path.join(OUT, "tsan")
    os.makedirs(out, exist_ok=True)
    exe = os.path.join(out, "serve_race")
    flags = ["g++", "-std=c++17", "-O1", "-g", "-fsanitize=thread", "-fPIC", "-pthread",
             "-I", cuda_include(), "-I", CSRC, "-I", HERE,
             "-I", os.path.join(ROOT, "include")]
    srcs = [os.path.join(CSRC, f) for f in HOST_UNITS] + [
        os.path.join(HERE, f) for f in SIM_UNITS + ["serve_race.cpp"]]
    if not _stale(exe, srcs + _deps() + [os.path.abspath(__file__)]):
        return exe
    objs = []

    def one(src):
        obj = os.path.join(out, os.path.basename(src).rsplit(".", 1)[0] + ".o")
        lang = ["-x", "c++"] if src.endswith(".cu") else []
        r = subprocess.run(flags + lang + ["-c", src, "-o", obj], capture_output=True,
                           text=True)
        if r.returncode != 0:
            raise RuntimeError("tsan build failed:\n%s" % r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(one, srcs))
    r = subprocess.run(["g++", "-fsanitize=thread", "-pthread", "-o", exe] + objs,
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("tsan link failed:\n%s" % r.stderr)
    return exe


if __name__ == "__main__":
    print(build())
    sys.exit(0)
