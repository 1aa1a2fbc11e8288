"""GPU test files run on the CPU against the host simulation of the device
side (``tests/harness/sim``).

libgbcc's host code is compiled for the host and linked against host models
of the kernel launchers and a stand-in CUDA runtime that emulates stream
capture. That code is:
- the C ABI;
- the CCSD driver with its CUDA-graph capture;
- the contraction engine;
- the complex and stored programs on the CUDA backend;
- serving.

The step runner, which links libgbcc.so, picks up the simulation through
LD_LIBRARY_PATH.

What this checks is the host code and every call it makes into the device
routines: argument order, shapes, buffer lifetimes, and what may run while a
stream is captured. The kernels themselves are checked on the GPU. The
calibration set consists of GPU tests that have already passed on a GB300.
Running it on the simulation shows that the models follow the kernels. The
runs below leave out tests that need torch device memory, bounded device
waits or GPU-sized workloads.
"""
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CALIBRATION = ["tests/test_gpu_parity.py", "tests/test_gpu_failure.py",
               "tests/test_gpu_serve.py", "-k",
               "not dgemm_all and not matrix_vector and not c1_config and not device_wait"
               " and not alone_equals and not requests_overlap"]
RUNNER = ["tests/test_gpu_runner.py"]
NEW_PATHS = ["tests/test_zzz_energy_terms.py", "tests/test_zzz_complex_branch.py",
             "tests/test_zzz_stored_formulation.py", "tests/test_zzz_golden_fixtures.py",
             "tests/test_zzz_solver_options.py", "tests/test_zzz_stepping_api.py",
             "tests/test_zzz_failure_new_paths.py", "tests/test_gpu_batch.py"]


@pytest.fixture(scope="module")
def sim_env():
    sys.path.insert(0, os.path.join(ROOT, "tests", "harness", "sim"))
    try:
        import build_sim
    finally:
        sys.path.pop(0)
    lib = build_sim.build()
    from sisi4s_gb300 import build
    build.build()  # the step runner binary
    env = dict(os.environ)
    env["GBCC_SIM_LIB"] = lib
    env["LD_LIBRARY_PATH"] = build_sim.LD_DIR + (
        ":" + env["LD_LIBRARY_PATH"] if env.get("LD_LIBRARY_PATH") else "")
    return env


def _pytest(env, args):
    r = subprocess.run([sys.executable, "-m", "pytest", "-m", "gpu", "-q", "-p",
                        "no:cacheprovider"] + args, cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=1200)
    assert r.returncode == 0, r.stdout[-6000:] + r.stderr[-2000:]
    return r.stdout


def test_simulated_capture_follows_cuda_rules(sim_env):
    """The stand-in runtime's stream capture: work is recorded, not run, and
    runs at every graph launch; synchronising calls and copies with pageable
    host memory are refused during the capture, as under CUDA."""
    import ctypes as C

    import numpy as np
    lib = C.CDLL(sim_env["GBCC_SIM_LIB"])
    vp = C.c_void_p
    s, dev, pinned, graph, exe = vp(), vp(), vp(), vp(), vp()
    assert lib.cudaStreamCreateWithFlags(C.byref(s), 1) == 0
    assert lib.cudaMallocAsync(C.byref(dev), C.c_size_t(64), s) == 0
    assert lib.cudaMallocHost(C.byref(pinned), C.c_size_t(64)) == 0
    buf = (C.c_ubyte * 64).from_address(pinned.value)
    C.memset(pinned, 0, 64)
    assert lib.cudaMemsetAsync(dev, 0, C.c_size_t(64), s) == 0
    assert lib.cudaStreamBeginCapture(s, 1) == 0
    assert lib.cudaMemsetAsync(dev, 7, C.c_size_t(64), s) == 0
    assert lib.cudaMemcpyAsync(pinned, dev, C.c_size_t(64), 2, s) == 0  # device to host
    assert lib.cudaStreamSynchronize(s) != 0
    assert lib.cudaMalloc(C.byref(vp()), C.c_size_t(8)) != 0
    host = np.zeros(8)
    assert lib.cudaMemcpyAsync(vp(host.ctypes.data), dev, C.c_size_t(64), 2, s) != 0
    assert lib.cudaStreamEndCapture(s, C.byref(graph)) == 0
    assert bytes(buf) == bytes(64)  # recorded, not run
    assert lib.cudaGraphInstantiate(C.byref(exe), graph, C.c_ulonglong(0)) == 0
    assert lib.cudaGraphDestroy(graph) == 0
    assert lib.cudaGraphLaunch(exe, s) == 0
    assert bytes(buf) == bytes([7] * 64)
    assert lib.cudaMemsetAsync(dev, 0, C.c_size_t(64), s) == 0
    assert lib.cudaGraphLaunch(exe, s) == 0  # runs again
    assert bytes(buf) == bytes([7] * 64)
    assert lib.cudaStreamSynchronize(s) == 0
    for call in (lib.cudaGraphExecDestroy(exe), lib.cudaFreeAsync(dev, s),
                 lib.cudaFreeHost(pinned), lib.cudaStreamDestroy(s)):
        assert call == 0


def test_calibration_set_passes_on_the_simulation(sim_env):
    out = _pytest(sim_env, CALIBRATION + RUNNER)
    assert " passed" in out and "failed" not in out


def test_newer_path_gpu_tests_pass_on_the_simulation(sim_env):
    out = _pytest(sim_env, NEW_PATHS)
    assert " passed" in out and "failed" not in out


def _runtime(name, compiler="gcc"):
    p = subprocess.run([compiler, "-print-file-name=" + name], capture_output=True,
                       text=True).stdout.strip()
    return p if os.path.isabs(p) and os.path.exists(p) else None


def test_host_code_under_address_and_undefined_behaviour_sanitizers(sim_env):
    """The library's host code, built with ASan and UBSan, through the new-path
    and calibration GPU test files on the simulation (the UEG complex-branch
    solve is left out for time).  Any report fails the run."""
    asan, cxx = _runtime("libasan.so"), _runtime("libstdc++.so.6", "g++")
    if not asan or not cxx:
        pytest.skip("the sanitizer runtime is not installed")
    sys.path.insert(0, os.path.join(ROOT, "tests", "harness", "sim"))
    try:
        import build_sim
    finally:
        sys.path.pop(0)
    lib, ld = build_sim.build_sanitized()
    env = dict(sim_env)
    env["GBCC_SIM_LIB"] = lib
    env["LD_LIBRARY_PATH"] = ld + ":" + sim_env["LD_LIBRARY_PATH"]
    # the library is loaded into Python: its runtimes must come first
    env["LD_PRELOAD"] = asan + " " + cxx
    env["ASAN_OPTIONS"] = "detect_leaks=0:halt_on_error=1"
    env["UBSAN_OPTIONS"] = "halt_on_error=1:print_stacktrace=1"
    # (the lockstep-batch files run on the plain simulation only, for time)
    args = [f for f in NEW_PATHS if f != "tests/test_gpu_batch.py"] + CALIBRATION[:-2] + RUNNER + [
        "-k", CALIBRATION[-1] + " and not ueg_golden_through_the_complex"]
    r = subprocess.run([sys.executable, "-m", "pytest", "-m", "gpu", "-q", "-p",
                        "no:cacheprovider"] + args, cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=1800)
    text = r.stdout + r.stderr
    assert "runtime error" not in text and "AddressSanitizer" not in text, text[-6000:]
    assert r.returncode == 0, text[-6000:]


def test_serving_threads_have_no_data_race():
    """gbcc_server's workers, queue and statistics under ThreadSanitizer."""
    sys.path.insert(0, os.path.join(ROOT, "tests", "harness", "sim"))
    try:
        import build_sim
    finally:
        sys.path.pop(0)
    exe = build_sim.build_serve_race()
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    if "unexpected memory mapping" in r.stderr:
        pytest.skip("ThreadSanitizer cannot run under this kernel's memory layout")
    assert "ThreadSanitizer" not in r.stderr, r.stderr[-4000:]
    assert r.returncode == 0, r.stdout + r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("id ")]
    assert len(lines) == 16 and all(" st 0 status 0 " in l for l in lines), r.stdout


@pytest.mark.parametrize("module,argv", [
    ("complex_bench", ["3", "8", "12", "--iterations", "3"]),
    ("solve_bench", ["3", "10", "24", "--iterations", "3", "--formulation", "stored",
                     "--triples-fp64-on-emu"]),
    ("solve_bench", ["3", "10", "24", "--iterations", "3"]),
])
def test_measurement_scripts_run_on_the_simulation(sim_env, module, argv):
    """The measurement scripts of the complex branch and of the two real
    formulations end to end (they need no torch)."""
    code = ("import os, sys, runpy; from sisi4s_gb300 import capi; "
            "capi.load(os.environ['GBCC_SIM_LIB']); "
            "sys.argv = [%r] + %r; "
            "runpy.run_module('benchmarks.%s', run_name='__main__')" % (module, argv, module))
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=sim_env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    import json
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["dE_ccsd_ha"] == 0.0  # FP64 products model both precisions here
    assert set(line["emu"]) >= {"energy", "seconds_per_iteration", "e_t"}


def test_smoke_entry_runs_on_the_simulation(sim_env):
    code = ("import os; from sisi4s_gb300 import capi; capi.load(os.environ['GBCC_SIM_LIB']); "
            "import __graft_entry__ as g; g.smoke()")
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=sim_env,
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "smoke ok" in r.stdout
