"""Seeded inputs behind the golden fixtures of this folder.

``make_golden.py`` runs the oracle on these inputs to write the fixtures, and
the fixture tests rebuild the same inputs to check the oracle (on the CPU) and
the GPU path against them.  No dataset is involved: every system comes from
``sisi4s_gb300.inputs.make_system`` (seeded normal vertex, uniform
eigenvalues); the complex one adds a seeded unitary rotation of the vertex
rows and seeded orbital phases, so that its integrals are complex while its
energies stay those of a physical system.
"""
import json
import os

import numpy as np

from sisi4s_gb300.inputs import make_system

HERE = os.path.dirname(os.path.abspath(__file__))

#: the reference's UEG integration test (7 holes, 26 particles, rs = 1.0)
UEG_FILE = os.path.join(HERE, "ueg_rs1.0-7occ-26virt.json")
#: the oracle's energies on REAL / COMPLEX below
ORACLE_FILE = os.path.join(HERE, "oracle_cases.json")

#: real closed-shell system: DIIS(5) from the MP2 start, a fixed number of
#: iterations (no convergence test stops it), in both formulations
REAL = {"No": 5, "Nv": 16, "NG": 40, "seed": 21}
REAL_SOLVE = {"mixer": "DiisMixer", "max_residua": 5, "max_iterations": 8,
              "energy_convergence": 0.0, "amplitudes_convergence": 0.0}

#: complex (k-point-like) system: linear mixer (the only complex mixer of the
#: reference), a fixed number of iterations, sliced ladder
COMPLEX = {"No": 3, "Nv": 9, "NG": 14, "seed": 6}
COMPLEX_SOLVE = {"mixing_ratio": 1.0, "max_iterations": 10, "energy_convergence": 0.0,
                 "amplitudes_convergence": 0.0, "slice_size": 2}

#: the headline workload: No=32, Nv=256, NG=1024 from seed 1, 12 iterations
#: from the MP2 start with DIIS(5) and a level shift of 16 Ha.  On this
#: generator the reference's default LinearMixer overflows within a few
#: iterations, and DIIS without a shift wanders chaotically (|E| ~ 1e6 Ha by
#: iteration 11, where two arithmetics differing at 1e-13 per step end up
#: 1e-4 Ha apart); the shift keeps the 12 iterations well conditioned, so an
#: energy difference between two arithmetics measures their own error.
C2 = {"No": 32, "Nv": 256, "NG": 1024, "seed": 1}
C2_SOLVE = {"mixer": "DiisMixer", "max_residua": 5, "level_shift": 16.0,
            "max_iterations": 12, "energy_convergence": 0.0,
            "amplitudes_convergence": 0.0}
#: FP64 energies of C2 (oracle trajectory, FP64 (T)); see make_c2_fixture.py
C2_FILE = os.path.join(HERE, "c2_trajectory.json")


def real_system():
    return make_system(**REAL)


def complex_system(No, Nv, NG, seed):
    """(system, complex vertex): make_system's vertex rotated by a unitary W
    over its rows and by orbital phases,
    Gamma'[G, p, q] = sum_H W[G, H] conj(ph_p) Gamma[H, p, q] ph_q."""
    s = make_system(No, Nv, NG, seed=seed)
    rng = np.random.default_rng(seed + 100)
    W, _ = np.linalg.qr(rng.normal(size=(NG, NG)) + 1j * rng.normal(size=(NG, NG)))
    ph = np.exp(1j * rng.uniform(0, 2 * np.pi, No + Nv))
    g = np.einsum("GH,Hpq->Gpq", W, np.conj(ph)[None, :, None] * s.gamma * ph[None, None, :])
    return s, g


def load(path):
    with open(path) as f:
        return json.load(f)


def complex_list(pairs):
    """[[re, im], ...] -> complex array"""
    a = np.asarray(pairs, dtype=np.float64)
    return a[:, 0] + 1j * a[:, 1]
