"""Oracle restatement of the sisi4s amplitude mixers.

Test infrastructure only (see ``oracle/__init__.py``).

Amplitudes are "Fock vectors": a tuple ``(T1, T2)``.  The reference's
``FockVector::dot`` (src/math/FockVector.hpp:226-236) is the sum over all
components of conj(x)*y; for real amplitudes it is the plain dot product.
"""
import numpy as np
import scipy.linalg.lapack as lapack

__all__ = ["fv_dot", "DiisMixer", "LinearMixer", "make_mixer", "DiisSingular"]


def fv_dot(x, y):
    """FockVector::dot for real (T1, T2) pairs: one reduction per component,
    summed in component order (src/math/FockVector.hpp:226-236)."""
    return float(np.dot(x[0].ravel(), y[0].ravel())) + float(
        np.dot(x[1].ravel(), y[1].ravel()))


class DiisSingular(RuntimeError):
    """dsysv reported info != 0 (src/mixers/DiisMixer.cxx:35-39)."""


def diis_inverse(matrix):
    """``inverse(matrix, N)`` of src/mixers/DiisMixer.cxx:16-41: solve
    B c = (-1, 0, ..., 0) with LAPACK dsysv on the upper triangle."""
    n = matrix.shape[0]
    rhs = np.zeros((n, 1))
    rhs[0, 0] = -1.0
    _, _, x, info = lapack.dsysv(np.asfortranarray(matrix), rhs, lower=0)
    if info != 0:
        raise DiisSingular("problem diagonalization (dsysv info=%d)" % info)
    return x[:, 0].copy()


class DiisMixer:
    """src/mixers/DiisMixer.cxx:50-186.

    B is (N+1)x(N+1) with B[0,1:] = B[1:,0] = -1 and B[0,0] = 0 (:68-96).
    ``append`` stores (A, R) at ``next_index``, writes the overlaps
    2*<R_i, R> into row and column next_index+1 (:115-140), solves the
    leading (count+1)^2 block (:145-151) and forms
    next = sum_j c_{i+1} A_i with i = (next_index + N - j) % N, j = 0..count-1,
    starting from a zero vector and adding one scaled term at a time
    (:160-174).
    """

    def __init__(self, max_residua=4):
        n = int(max_residua)
        self.N = n
        self.amplitudes = [None] * n
        self.residua = [None] * n
        self.next_index = 0
        self.count = 0
        self.B = np.zeros((n + 1, n + 1))
        self.B[0, 1:] = -1.0
        self.B[1:, 0] = -1.0
        self.next = None
        self.next_residuum = None
        self.last_weights = None
        self.last_lambda = None

    def append(self, A, R):
        n = self.N
        k = self.next_index
        self.amplitudes[k] = A
        self.residua[k] = R
        for i in range(n):
            if self.residua[i] is not None:
                overlap = 2.0 * fv_dot(self.residua[i], R)
                self.B[k + 1, i + 1] = overlap
                if i == k:
                    continue
                self.B[i + 1, k + 1] = overlap
        if self.count < n:
            self.count += 1
        dim = self.count + 1
        column = diis_inverse(self.B[:dim, :dim].copy())
        self.last_lambda = column[0]
        nxt = [np.zeros_like(A[0]), np.zeros_like(A[1])]
        nres = [np.zeros_like(R[0]), np.zeros_like(R[1])]
        weights = []
        for j in range(self.count):
            i = (k + n - j) % n
            c = column[i + 1]
            weights.append(c)
            for comp in range(2):
                nxt[comp] = nxt[comp] + c * self.amplitudes[i][comp]
                nres[comp] = nres[comp] + c * self.residua[i][comp]
        self.last_weights = weights
        self.next = (nxt[0], nxt[1])
        self.next_residuum = (nres[0], nres[1])
        self.next_index = (k + 1) % n

    def get(self):
        return self.next


class LinearMixer:
    """src/mixers/LinearMixer.cxx:12-54.  With ``ratio`` 1 this is plain
    Jacobi.  Note that ``append`` scales the caller's ``next`` and
    ``nextResiduum`` in place, so the driver's amplitude-change vector (used in
    the convergence test) is the mixed one."""

    def __init__(self, ratio=1.0):
        self.ratio = float(ratio)
        self.last = None
        self.last_residuum = None

    def append(self, nxt, nres):
        # in-place semantics: nxt / nres are lists so that the caller sees
        # the scaled values, as with the reference's shared pointers
        if self.last is not None:
            r = self.ratio
            for comp in range(2):
                self.last[comp] = self.last[comp] * (1 - r)
                nxt[comp] = nxt[comp] * r
                nxt[comp] = nxt[comp] + self.last[comp]
                self.last_residuum[comp] = self.last_residuum[comp] * (1 - r)
                nres[comp] = nres[comp] * r
                nres[comp] = nres[comp] + self.last_residuum[comp]
        self.last = nxt
        self.last_residuum = nres

    def get(self):
        return (self.last[0], self.last[1])


def make_mixer(name="LinearMixer", max_residua=4, mixing_ratio=1.0):
    """MixerFactory::create (src/mixers/Mixer.hpp:54-93)."""
    if name == "DiisMixer":
        return DiisMixer(max_residua)
    if name == "LinearMixer":
        return LinearMixer(mixing_ratio)
    raise ValueError("Mixer not implemented: %s" % name)
