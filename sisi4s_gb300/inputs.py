"""Seeded synthetic CCSD(T) systems.

No public dataset is involved: the workloads are random closed-shell systems
with the shapes and value distributions below.  For a seed:

* the vertex Gamma[G, p, q] (holes p < No first, then particles) has, for every
  G, its upper triangle (diagonal included, row-major order) drawn from
  N(0, 0.03^2) and mirrored, so Gamma_pq = Gamma_qp and every element is
  exactly N(0, 0.03^2).  All NG rows are drawn in one call, before anything
  else;
* hole eigenvalues eps_i ~ U[-1.5, -0.5], then particle eigenvalues
  eps_a ~ U[0.2, 3.0], each sorted ascending.

The generator is ``numpy.random.default_rng(seed)``.  Arrays are returned
with the reference's index order; ``to_device_layout`` gives the column-major
(first index fastest) flat buffers that the C ABI takes.
"""
from dataclasses import dataclass

import numpy as np

__all__ = ["System", "make_system", "column_major"]


@dataclass
class System:
    No: int
    Nv: int
    NG: int
    gamma: np.ndarray   # [NG, Np, Np]
    eps_h: np.ndarray   # [No]
    eps_p: np.ndarray   # [Nv]
    seed: int

    @property
    def Np(self):
        return self.No + self.Nv


def make_system(No, Nv, NG, seed=1):
    rng = np.random.default_rng(seed)
    Np = No + Nv
    iu = np.triu_indices(Np)
    vals = rng.normal(0.0, 0.03, size=(NG, iu[0].size))
    # column-major (first index fastest), the layout CTF hands to the
    # reference's algorithms, so the ABI wrappers pass it without a copy
    gamma = np.empty((NG, Np, Np), dtype=np.float64, order="F")
    gamma[:, iu[0], iu[1]] = vals
    gamma[:, iu[1], iu[0]] = vals
    eps_h = np.sort(rng.uniform(-1.5, -0.5, size=No))
    eps_p = np.sort(rng.uniform(0.2, 3.0, size=Nv))
    return System(No, Nv, NG, gamma, eps_h, eps_p, seed)


def column_major(a):
    """Flat float64 buffer of ``a`` with the first index fastest, the layout
    of CTF dense storage and of the cc4s ``.elements`` files."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).transpose(
        tuple(range(a.ndim - 1, -1, -1)))).ravel()


def mp2_amplitudes(system):
    """MP2 amplitudes T2 = -V_abij / D_abij (T1 = 0) in the reference's index
    order: the amplitudes the MP2-start iteration produces, used as given
    starting amplitudes.  V_abij = sum_G Gamma_Gai Gamma_Gbj."""
    No = system.No
    gai = system.gamma[:, No:, :No]
    v = np.einsum("Gai,Gbj->abij", gai, gai, optimize=True)
    ep, eh = system.eps_p, system.eps_h
    d = (((ep[:, None, None, None] - eh[None, None, :, None]) + ep[None, :, None, None])
         - eh[None, None, None, :])
    return np.zeros((system.Nv, No), order="F"), np.asfortranarray(-v / d)
