"""Builds libgbcc.so (CUDA kernels + C ABI) and the sisi4s-gb300 host runner
in-tree with nvcc for sm_103a.

Translation units compile in parallel; the result lands in
``sisi4s_gb300/_lib/``.  A unit is recompiled only when it or a header is
newer than its object file.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT = os.path.join(HERE, "_lib")
OBJ = os.path.join(OUT, "obj")
LIB = os.path.join(OUT, "libgbcc.so")
RUNNER = os.path.join(OUT, "sisi4s-gb300")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-Wall", "--expt-relaxed-constexpr",
              "-Xptxas", "-warn-spills"] + ARCH


def nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc",
                 shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _headers(d):
    return [os.path.join(d, f) for f in os.listdir(d)
            if f.endswith((".hpp", ".h", ".cuh"))] + [
        os.path.join(ROOT, "include", "gbcc.h")]


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def build(verbose=False, jobs=None):
    os.makedirs(OBJ, exist_ok=True)
    cc = nvcc()
    srcs = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    hdrs = _headers(CSRC)
    objs = []
    todo = []
    for s in srcs:
        src = os.path.join(CSRC, s)
        obj = os.path.join(OBJ, s[:-3] + ".o")
        objs.append(obj)
        if _stale(obj, [src] + hdrs):
            todo.append([cc] + NVCC_FLAGS + ["-c", src, "-o", obj])
    jobs = jobs or min(len(todo) or 1, os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        for out in ex.map(_run, todo):
            if verbose and out.strip():
                print(out)
    if todo or not os.path.exists(LIB):
        _run([cc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    # host runner (C++17, links the library)
    if os.path.isdir(HOST):
        hsrc = sorted(os.path.join(HOST, f) for f in os.listdir(HOST)
                      if f.endswith(".cpp"))
        if hsrc and _stale(RUNNER, hsrc + _headers(HOST) + [LIB]):
            _run(["g++", "-O2", "-std=c++17", "-Wall", "-I",
                  os.path.join(ROOT, "include"), "-o", RUNNER] + hsrc +
                 ["-L", OUT, "-lgbcc", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
