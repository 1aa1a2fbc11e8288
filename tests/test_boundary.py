"""The drop-in boundary without a GPU: the C ABI exports, the YAML step runner
(parsing, data symbols, cc4s tensor files, fallible steps)."""
import json
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(ROOT, "sisi4s_gb300", "_lib", "libgbcc.so")
RUNNER = os.path.join(ROOT, "sisi4s_gb300", "_lib", "sisi4s-gb300")


@pytest.fixture(scope="module", autouse=True)
def built():
    from sisi4s_gb300 import build
    build.build()


def declared_functions():
    text = open(os.path.join(ROOT, "include", "gbcc.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(gbcc_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_function():
    out = subprocess.run(["nm", "-D", "--defined-only", LIB], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\b(gbcc_[a-z0-9_]+)\b", out))
    decl = declared_functions()
    assert len(decl) >= 20
    missing = [f for f in decl if f not in exported]
    assert not missing, missing


def test_library_loads_and_reports_no_device_without_gpu():
    import ctypes
    from sisi4s_gb300 import capi
    lib = capi.load()
    assert lib.gbcc_abi_version() == 1
    assert lib.gbcc_status_string(capi.TIMEOUT) == b"TIMEOUT"
    h = ctypes.c_void_p()
    st = lib.gbcc_ctx_create(0, None, ctypes.byref(h))
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if not has_gpu:
        assert st == capi.NO_DEVICE
    else:
        assert st == capi.OK
        lib.gbcc_ctx_destroy(h)


def _run(tmp_path, yaml_text, *extra):
    inp = tmp_path / "in.yaml"
    inp.write_text(yaml_text)
    out = tmp_path / "out.yaml"
    r = subprocess.run([RUNNER, "-i", str(inp), "-o", str(out), "-l",
                        str(tmp_path / "log"), *extra], cwd=tmp_path,
                       capture_output=True, text=True)
    return r, json.loads(out.read_text())


def _write_tensor(path, arr, binary=True):
    flat = np.asarray(arr, dtype=np.float64).transpose(
        tuple(range(arr.ndim - 1, -1, -1))).ravel()
    dims = "".join("  - length: %d\n    type: State\n" % n for n in arr.shape)
    path.write_text("version: 100\ntype: Tensor\ndimensions:\n%sscalarType: Real64\n"
                    "elements:\n  type: %s\nunit: 1.0\n"
                    % (dims, "IeeeBinaryFile" if binary else "TextFile"))
    ep = str(path)[:-5] + ".elements"
    if binary:
        flat.tofile(ep)
    else:
        np.savetxt(ep, flat, fmt="%.17g")


def test_read_write_roundtrip_and_symbols(tmp_path):
    rng = np.random.default_rng(0)
    a = rng.normal(size=(3, 4, 5))
    _write_tensor(tmp_path / "A.yaml", a, binary=True)
    _write_tensor(tmp_path / "B.yaml", a[0], binary=False)
    r, out = _run(tmp_path, """
- name: Nop    # anchors as in the reference's inputs
  energyConvergence: &ec 1e-8
  mixer: &mx DiisMixer
- name: Read
  in:
    fileName: "A.yaml"
  out:
    destination: $A
- name: Read
  in: { fileName: B.yaml }
  out: { destination: $B }
- name: Write
  in:
    source: $A
    fileName: "C.yaml"
  out: {}
- name: TensorWriter
  in:  { Data: $B }
  out:
    {}
- name: Nop
  in:
    a: *ec
    b: *mx
    c: 3
    d: $Undefined
""")
    assert r.returncode == 0, r.stderr
    back = np.fromfile(tmp_path / "C.elements").reshape(5, 4, 3).transpose(2, 1, 0)
    assert np.array_equal(back, a)
    lines = (tmp_path / "B.dat").read_text().split("\n")
    assert lines[0] == "B 2 4 5" and lines[1] == "ij "   # name order lens; row / column orders
    txt = np.array([float(x) for x in lines[2:] if x])
    assert np.allclose(txt, a[0].T.ravel(), rtol=1e-15, atol=0)
    last = out["steps"][-1]["in"]
    assert last["a"] == 1e-8 and last["b"] == "DiisMixer" and last["c"] == 3
    assert last["d"] == "Undefined"


def test_define_holes_and_particles(tmp_path):
    (tmp_path / "E.yaml").write_text(
        "metaData:\n  fermiEnergy: -0.1\n  energies: [-1.0, -0.5, 0.3, 0.9, 1.7]\n")
    r, out = _run(tmp_path, """
- name: DefineHolesAndParticles
  in:
    fileName: "E.yaml"
  out:
    HoleEigenEnergies: $Eh
    ParticleEigenEnergies: $Ep
- name: Write
  in: { source: $Eh, fileName: Eh.yaml }
- name: Write
  in: { source: $Ep, fileName: Ep.yaml }
""")
    assert r.returncode == 0, r.stderr
    assert out["steps"][0]["No"] == 2 and out["steps"][0]["Nv"] == 3
    assert np.array_equal(np.fromfile(tmp_path / "Eh.elements"), [-1.0, -0.5])
    assert np.array_equal(np.fromfile(tmp_path / "Ep.elements"), [0.3, 0.9, 1.7])


def test_dry_run_of_full_ccsd_t_input(tmp_path):
    r, out = _run(tmp_path, """
- name: Nop
  maxIterations: &maxIterations 50
- name: CcsdEnergyFromCoulombIntegrals
  in:
    mixer: DiisMixer
    maxResidua: 4
    maxIterations: *maxIterations
    energyConvergence: 1e-8
    CoulombVertex: $CoulombVertex
    HoleEigenEnergies: $HoleEigenEnergies
    ParticleEigenEnergies: $ParticleEigenEnergies
  out:
    CcsdEnergy: $CcsdEnergy
    CcsdSinglesAmplitudes: $T1
    CcsdDoublesAmplitudes: $T2
- name: CcsdPerturbativeTriples
  in:
    CoulombVertex: $CoulombVertex
    CcsdEnergy: $CcsdEnergy
    CcsdSinglesAmplitudes: $T1
    CcsdDoublesAmplitudes: $T2
    HoleEigenEnergies: $HoleEigenEnergies
    ParticleEigenEnergies: $ParticleEigenEnergies
  out:
    CcsdPerturbativeTriplesEnergy: $E
""", "--dry")
    assert r.returncode == 0, r.stderr
    assert [s["name"] for s in out["steps"]] == [
        "Nop", "CcsdEnergyFromCoulombIntegrals", "CcsdPerturbativeTriples"]
    assert out["steps"][1]["in"]["maxIterations"] == 50


def test_unknown_algorithm_and_fallible(tmp_path):
    r, out = _run(tmp_path, "- name: NoSuchAlgorithm\n")
    assert r.returncode == 1 and "unknown algorithm" in out["error"]
    r, out = _run(tmp_path, """
- name: Read
  fallible: true
  in: { fileName: missing.yaml }
  out: { destination: $X }
- name: Nop
""")
    assert r.returncode == 0
    assert "failed" in out["steps"][0] and out["steps"][1]["name"] == "Nop"


def test_list_algorithms():
    r = subprocess.run([RUNNER, "--list"], capture_output=True, text=True, check=True)
    names = r.stdout.split()
    for n in ("CcsdEnergyFromCoulombIntegrals", "CcsdPerturbativeTriples",
              "CcsdPerturbativeTriplesComplex",
              "CoulombIntegralsFromVertex", "Read", "Write", "TensorWriter", "TensorReader",
              "DefineHolesAndParticles", "Nop"):
        assert n in names


def _read_steps(names):
    return "".join("- name: Read\n  in: { fileName: %s.yaml }\n  out: { destination: $%s }\n"
                   % (n, n) for n in names)


@pytest.mark.parametrize("step,bad,msg", [
    ("CcsdPerturbativeTriples", None, None),
    ("CcsdPerturbativeTriples", "T2",
     "CcsdDoublesAmplitudes has lengths [3,3,2,3], expected [3,3,2,2]"),
    ("CcsdEnergyFromCoulombIntegrals", "V",
     "PPHHCoulombIntegrals has lengths [3,3,2,3], expected [3,3,2,2]"),
    ("CcsdEnergyFromCoulombIntegrals", "F", "HPFockMatrix has lengths [2,4], expected [2,3]"),
    ("CcsdEnergyFromCoulombIntegralsReference", None, None),
    ("CcsdEnergyFromCoulombIntegralsReference", "P4",
     "PPPPCoulombIntegrals has lengths [3,3,3,4], expected [3,3,3,3]"),
])
def test_tensor_lengths_are_checked_before_the_library_is_called(tmp_path, step, bad, msg):
    # the C ABI takes bare pointers: a tensor of the wrong lengths must be
    # refused by the runner, not read past its end
    rng = np.random.default_rng(1)
    No, Nv, NG = 2, 3, 4
    good = {"Eh": (No,), "Ep": (Nv,), "G": (NG, No + Nv, No + Nv), "T1": (Nv, No),
            "T2": (Nv, Nv, No, No), "V": (Nv, Nv, No, No), "F": (No, Nv),
            "P4": (Nv, Nv, Nv, Nv), "P3": (Nv, Nv, Nv, No)}
    for n, shape in good.items():
        if n == bad:
            shape = shape[:-1] + (shape[-1] + 1,)
        # a well-posed system, so that on a device the step also succeeds:
        # holes below particles, small integrals and amplitudes
        x = {"Eh": -1.0 - rng.uniform(size=shape), "Ep": 1.0 + rng.uniform(size=shape)}.get(
            n, 0.05 * rng.normal(size=shape))
        _write_tensor(tmp_path / ("%s.yaml" % n), x)
    out_keys = {"CcsdPerturbativeTriples": "{ CcsdPerturbativeTriplesEnergy: $E }"}
    r, out = _run(tmp_path, _read_steps(good) + """
- name: %s
  in:
    CoulombVertex: $G
    HoleEigenEnergies: $Eh
    ParticleEigenEnergies: $Ep
    PPHHCoulombIntegrals: $V
    PPPPCoulombIntegrals: $P4
    PPPHCoulombIntegrals: $P3
    HPFockMatrix: $F
    CcsdEnergy: 0.0
    CcsdSinglesAmplitudes: $T1
    CcsdDoublesAmplitudes: $T2
  out: %s
""" % (step, out_keys.get(step, "{}")))
    if bad is None:  # right lengths: the step reaches the library
        assert r.returncode == 0 or "GPU context: NO_DEVICE" in out["error"], out
        return
    assert r.returncode == 1
    assert msg in out["error"], out["error"]


@pytest.mark.parametrize("header,msg", [
    ("dimensions:\n  - type: State\nelements:\n  type: TextFile\n", "a dimension has no length"),
    ("dimensions:\n  - length: -2\nelements:\n  type: TextFile\n", "bad dimension length -2"),
    ("dimensions:\n  - length: 4294967296\n  - length: 4294967296\nelements:\n  type: TextFile\n",
     "bad dimension length 4294967296"),
    ("dimensions: 3\nelements:\n  type: TextFile\n", "dimensions must be a list"),
    ("dimensions:\n  - length: 2\nelements: TextFile\n", "elements.type missing"),
])
def test_malformed_tensor_headers_are_errors(tmp_path, header, msg):
    (tmp_path / "X.yaml").write_text("version: 100\ntype: Tensor\n" + header +
                                     "scalarType: Real64\nunit: 1\n")
    (tmp_path / "X.elements").write_text("1\n2\n")
    r, out = _run(tmp_path, _read_steps(["X"]))
    assert r.returncode == 1
    assert msg in out["error"], out["error"]


def test_ctypes_structs_match_the_c_header(tmp_path):
    """Every struct the Python binding mirrors has the C header's size and
    field offsets (compiled with the host C compiler)."""
    from sisi4s_gb300 import capi
    from sisi4s_gb300.serve import Result, ServerOpts
    mirrors = {"gbcc_ccsd_opts": capi.CcsdOpts, "gbcc_ccsd_in": capi.CcsdIn,
               "gbcc_ccsd_out": capi.CcsdOut, "gbcc_triples_in": capi.TriplesIn,
               "gbcc_ccsd_complex_in": capi.ComplexIn,
               "gbcc_ccsd_complex_out": capi.ComplexOut,
               "gbcc_triples_complex_in": capi.TriplesComplexIn,
               "gbcc_server_opts": ServerOpts, "gbcc_result": Result}
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbcc.h"',
             'int main(void) {']
    for cname, py in mirrors.items():
        lines.append('printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('printf("%s %s %%zu\\n", offsetof(%s, %s));'
                         % (cname, f, cname, f))
    lines += ['return 0;', '}']
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True, capture_output=True, text=True)
    got = {}
    for line in subprocess.run([str(exe)], check=True, capture_output=True,
                               text=True).stdout.split("\n"):
        if line:
            name, field, value = line.split()
            got[(name, field)] = int(value)
    import ctypes
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def _write_complex_tensor(path, arr):
    z = np.ascontiguousarray(np.asarray(arr, dtype=np.complex128).transpose(
        tuple(range(arr.ndim - 1, -1, -1)))).ravel()
    dims = "".join("  - length: %d\n    type: State\n" % n for n in arr.shape)
    path.write_text("version: 100\ntype: Tensor\ndimensions:\n%sscalarType: Complex64\n"
                    "elements:\n  type: IeeeBinaryFile\nunit: 1.0\n" % dims)
    z.view(np.float64).tofile(str(path)[:-5] + ".elements")


def test_complex_branch_is_chosen_by_the_integrals(tmp_path):
    # as in the reference (ClusterSinglesDoublesAlgorithm.cxx:25-35), complex
    # PPHH integrals select the complex branch; a complex vertex alone is read
    # by the real path as Re.Re + Im.Im; the real (T) refuses complex amplitudes
    rng = np.random.default_rng(2)
    No, Nv, NG = 2, 3, 4
    # a well-posed system, so that on a device the steps also succeed: holes
    # below particles, small integrals and amplitudes
    _write_tensor(tmp_path / "Eh.yaml", -1.0 - rng.uniform(size=No))
    _write_tensor(tmp_path / "Ep.yaml", 1.0 + rng.uniform(size=Nv))
    _write_tensor(tmp_path / "F.yaml", 0.05 * rng.normal(size=(No, Nv)))
    c = lambda *shape: 0.05 * (rng.normal(size=shape) + 1j * rng.normal(size=shape))
    _write_complex_tensor(tmp_path / "G.yaml", c(NG, No + Nv, No + Nv))
    _write_complex_tensor(tmp_path / "V.yaml", c(Nv, Nv, No, No))
    _write_complex_tensor(tmp_path / "T1.yaml", c(Nv, No))
    _write_tensor(tmp_path / "T2.yaml", 0.05 * rng.normal(size=(Nv, Nv, No, No)))
    reads = _read_steps(["Eh", "Ep", "F", "G", "V", "T1", "T2"])
    common = """    CoulombVertex: $G
    HoleEigenEnergies: $Eh
    ParticleEigenEnergies: $Ep
"""
    reaches_library = lambda r, out: r.returncode == 0 or "GPU context: NO_DEVICE" in out["error"]
    # every output a step sets is listed, as the reference requires
    # (Algorithm.cxx:37-45 throws on a missing argument)
    step = lambda name, extra, outs: (reads + "- name: %s\n  in:\n" % name + common + extra
                                      + "  out: { %s }\n" % outs)
    e = "CcsdEnergy: $E"
    r, out = _run(tmp_path, step("CcsdEnergyFromCoulombIntegrals",
                                 "    HPFockMatrix: $F\n    PPHHCoulombIntegrals: $V\n", e))
    assert reaches_library(r, out), out    # the complex branch with its Fock term
    r, out = _run(tmp_path, step("CcsdEnergyFromCoulombIntegrals",
                                 "    PPHHCoulombIntegrals: $V\n", e + ", PairEnergy: $P"))
    assert reaches_library(r, out), out
    r, out = _run(tmp_path, step("CcsdEnergyFromCoulombIntegralsReference",
                                 "    PPHHCoulombIntegrals: $V\n", e))
    assert r.returncode == 1 and "has a complex branch here" in out["error"], out
    r, out = _run(tmp_path, step("CcsdEnergyFromCoulombIntegrals", "    HPFockMatrix: $F\n", e))
    assert reaches_library(r, out), out
    amps = "    CcsdEnergy: 0.0\n    CcsdSinglesAmplitudes: $T1\n    CcsdDoublesAmplitudes: $T2\n"
    r, out = _run(tmp_path, step("CcsdPerturbativeTriples", amps,
                                 "CcsdPerturbativeTriplesEnergy: $Et"))
    assert r.returncode == 1 and "CcsdPerturbativeTriplesComplex" in out["error"], out
    r, out = _run(tmp_path, step("CcsdPerturbativeTriplesComplex", amps,
                                 "CcsdPerturbativeTriplesComplexEnergy: $Et"))
    assert reaches_library(r, out), out
    r, out = _run(tmp_path, step("CoulombIntegralsFromVertex", "    complex: 1\n",
                                 "PPHHCoulombIntegrals: $W"))
    assert reaches_library(r, out), out


def test_tensor_writer_and_reader_formats(tmp_path):
    """TensorWriter / TensorReader in the formats of src/util/TensorIo.cxx and
    src/util/BinaryTensorFormat.hpp: text with a header line, index-order line
    and row x column layout; binary with a 32-byte header and 8 bytes per
    dimension."""
    import struct
    rng = np.random.default_rng(4)
    a = rng.normal(size=(3, 4, 5))
    z = rng.normal(size=(2, 3)) + 1j * rng.normal(size=(2, 3))
    _write_tensor(tmp_path / "A.yaml", a)
    _write_complex_tensor(tmp_path / "Z.yaml", z)
    r, out = _run(tmp_path, _read_steps(["A", "Z"]) + """
- name: TensorWriter
  in: { Data: $A, rowIndexOrder: jk, columnIndexOrder: i }
- name: TensorWriter
  in: { Data: $A, mode: binary }
- name: TensorWriter
  in: { Data: $Z, file: Z.dat }
- name: TensorWriter
  in: { Data: $Z, mode: binary, file: Z.bin }
- name: TensorReader
  in: { file: A.dat }
  out: { Data: $At }
- name: TensorReader
  in: { mode: binary, file: A.bin }
  out: { Data: $Ab }
- name: TensorReader
  in: { file: Z.dat, complexVersion: 1 }
  out: { Data: $Zt }
- name: TensorReader
  in: { mode: binary, file: Z.bin, complexVersion: 1 }
  out: { Data: $Zb }
- name: Write
  in: { source: $At, fileName: At.yaml }
- name: Write
  in: { source: $Ab, fileName: Ab.yaml }
- name: Write
  in: { source: $Zt, fileName: Zt.yaml }
- name: Write
  in: { source: $Zb, fileName: Zb.yaml }
""")
    assert r.returncode == 0, (r.stderr, out)
    # text: one line per (j, k) row, j fastest; the i column values in order
    lines = (tmp_path / "A.dat").read_text().split("\n")
    assert lines[0] == "A 3 3 4 5" and lines[1] == "jk i"
    rows = [list(map(float, x.split(" "))) for x in lines[2:] if x]
    want = [[a[i, j, k] for i in range(3)] for k in range(5) for j in range(4)]
    assert np.allclose(rows, want, rtol=1e-15, atol=0)
    # binary: header, dimension headers, then first-index-fastest data
    raw = (tmp_path / "A.bin").read_bytes()
    assert struct.unpack("<4si4siiiii", raw[:32]) == (b"TENS", 0x9000, b"IEEE", 8, 1, 3, 0, 0)
    dims = [struct.unpack("<icbh", raw[32 + 8 * d:40 + 8 * d]) for d in range(3)]
    assert dims == [(3, b"a", 0, 0), (4, b"b", 0, 0), (5, b"c", 0, 0)]
    assert np.array_equal(np.frombuffer(raw[56:]), a.transpose(2, 1, 0).ravel())
    zraw = (tmp_path / "Z.bin").read_bytes()
    assert struct.unpack("<4si4siiiii", zraw[:32])[3:6] == (16, 2, 2)
    assert np.array_equal(np.frombuffer(zraw[48:]).view(np.complex128), z.T.ravel())
    zl = (tmp_path / "Z.dat").read_text().split("\n")
    assert zl[0] == "Z 2 2 3" and zl[2].startswith("(") and "," in zl[2]
    # the readers give the tensors back (the binary ones bit for bit)
    back = lambda n, shape: np.fromfile(tmp_path / (n + ".elements")).reshape(
        tuple(reversed(shape))).transpose(tuple(range(len(shape) - 1, -1, -1)))
    assert np.array_equal(back("Ab", a.shape), a)
    assert np.allclose(back("At", a.shape), a, rtol=1e-15, atol=0)
    zb = np.fromfile(tmp_path / "Zb.elements").view(np.complex128).reshape(3, 2).T
    zt = np.fromfile(tmp_path / "Zt.elements").view(np.complex128).reshape(3, 2).T
    assert np.array_equal(zb, z) and np.allclose(zt, z, rtol=1e-15, atol=0)


def test_yaml_subset_of_the_step_files(tmp_path):
    """The YAML the reference's step files use: comments (also after values,
    not inside quotes), anchors and aliases, flow maps and sequences, quoted
    scalars, enable / disable, and typed anonymous constants."""
    r, out = _run(tmp_path, """
# leading comment
- name: Nop            # trailing comment
  in:
    text: "a # not a comment"
    single: 'x: y'
    int: 42
    neg: -7
    real: 2.5e-3
    word: DiisMixer
    anchored: &anc 17
    alias: *anc
- name: Nop
  disable: true
  in: { never: 1 }
- name: Nop
  enable: false
- name: Nop
  in: {flow: 3, other: "q,r"}
  note: "kept"
""")
    assert r.returncode == 0, (r.stderr, out)
    steps = out["steps"]
    assert len(steps) == 2                      # the disabled steps are skipped
    first = steps[0]["in"]
    assert first["text"] == "a # not a comment" and first["single"] == "x: y"
    assert first["int"] == 42 and first["neg"] == -7 and first["real"] == 2.5e-3
    assert first["word"] == "DiisMixer" and first["alias"] == 17
    assert steps[1]["in"] == {"flow": 3, "other": "q,r"} and steps[1]["note"] == "kept"
