"""Host-side argument checks of the Python front end (no GPU).

The C ABI takes bare pointers and sizes, so the front end refuses arrays of
the wrong shape before anything reaches the library.  A complex vertex is
not dropped to its real part in a float64 cast: the real path reads it as
the reference's real CCSD does, Re.Re + Im.Im, i.e. as the real vertex with
the imaginary rows stacked under the real ones.
"""
import numpy as np
import pytest

from sisi4s_gb300 import ccsd as gpu
from sisi4s_gb300.inputs import make_system

No, Nv, NG = 2, 5, 7


@pytest.fixture(scope="module")
def system():
    return make_system(No, Nv, NG, seed=3)


def test_real_vertex_passes_no_imaginary_part(system):
    inp = gpu.CcsdInput(system.eps_h, system.eps_p, system.gamma)
    assert not inp.s.gamma_imag
    assert (inp.No, inp.Nv, inp.NG) == (No, Nv, NG)
    zero_im = gpu.CcsdInput(system.eps_h, system.eps_p, system.gamma.astype(complex))
    assert zero_im.NG == NG and np.array_equal(zero_im._keep[2], inp._keep[2])


def test_complex_vertex_is_stacked_for_the_real_path(system):
    g = system.gamma.astype(np.complex128)
    g[1, 2, 3] += 1e-3j
    inp = gpu.CcsdInput(system.eps_h, system.eps_p, g)
    assert not inp.s.gamma_imag and inp.NG == 2 * NG and inp.s.NG == 2 * NG
    # column-major [Re; Im]: element (G', p, q) at G' + p*2NG + q*2NG*Np
    Np = No + Nv
    flat = inp._keep[2]
    assert flat[NG + 1 + 2 * (2 * NG) + 3 * (2 * NG) * Np] == 1e-3
    assert flat[1 + 2 * (2 * NG) + 3 * (2 * NG) * Np] == g[1, 2, 3].real


def test_stacked_vertex_is_the_reference_real_path():
    # the oracle's real residual reads a complex vertex as Re.Re + Im.Im
    # (CcsdEnergyFromCoulombIntegrals.cxx:80-115); so does the stacked vertex
    from oracle.ccsd import residual
    from oracle.coulomb import coulomb_integrals
    s = make_system(No, Nv, NG, seed=7)
    rng = np.random.default_rng(8)
    g = s.gamma + 1j * 0.02 * rng.normal(size=s.gamma.shape)
    stacked = np.concatenate([g.real, g.imag], axis=0)
    T1 = rng.normal(0, 0.05, (Nv, No))
    T2 = rng.normal(0, 0.05, (Nv, Nv, No, No))
    T2 = 0.5 * (T2 + T2.transpose(1, 0, 3, 2))
    a = residual(1, T1, T2, coulomb_integrals(g, No), g, slice_size=2)
    b = residual(1, T1, T2, coulomb_integrals(stacked, No), stacked, slice_size=2)
    for x, y in zip(a, b):
        assert np.abs(x - y).max() < 1e-14 * np.abs(y).max()


@pytest.mark.parametrize("key,shape", [("PPHH", (Nv, Nv, No, No + 1)),
                                       ("PHPH", (Nv, Nv, No, No)),
                                       ("HHHH", (No, No, No)),
                                       ("HHHP", (No, No, No, No))])
def test_integrals_of_the_wrong_shape_are_refused(system, key, shape):
    with pytest.raises(ValueError, match=key):
        gpu.CcsdInput(system.eps_h, system.eps_p, system.gamma,
                      ints={key: np.zeros(shape)})


def test_bad_vertex_and_amplitudes_are_refused(system):
    with pytest.raises(ValueError, match="gamma"):
        gpu.CcsdInput(system.eps_h, system.eps_p, system.gamma[:, :-1, :])
    with pytest.raises(ValueError, match="eps_h"):
        gpu.CcsdInput(system.eps_h[:, None], system.eps_p, system.gamma)
    with pytest.raises(ValueError, match="initial T2"):
        gpu.CcsdInput(system.eps_h, system.eps_p, system.gamma,
                      initial=(np.zeros((Nv, No)), np.zeros((Nv, No, Nv, No))))
    with pytest.raises(ValueError, match="T1"):
        gpu.triples(None, system.eps_h, system.eps_p, system.gamma,
                    np.zeros((No, Nv)), np.zeros((Nv, Nv, No, No)))
    with pytest.raises(ValueError, match="No must"):
        gpu.coulomb_integrals(None, system.gamma, No + Nv)


def test_complex_front_end_layout_and_checks(system):
    g = system.gamma.astype(complex)
    g[2, 1, 4] += 0.5j
    inp = gpu.ComplexInput(system.eps_h, system.eps_p, g)
    # interleaved (re, im), first index fastest: element (G, p, q) at
    # 2 * (G + p*NG + q*NG*Np)
    Np = No + Nv
    e = 2 + 1 * NG + 4 * NG * Np
    assert inp._keep[2][2 * e + 1] == 0.5 and inp._keep[2][2 * e] == g[2, 1, 4].real
    with pytest.raises(ValueError, match="gamma"):
        gpu.ComplexInput(system.eps_h, system.eps_p, g[:, :-1, :])
    with pytest.raises(ValueError, match="initial T2"):
        gpu.ComplexInput(system.eps_h, system.eps_p, g,
                         initial=(np.zeros((Nv, No)), np.zeros((Nv, Nv, No))))
    z = (np.arange(6) + 1j * np.arange(6)).reshape(2, 3)
    assert np.array_equal(gpu.from_complex_flat(gpu.complex_flat(z, (2, 3), "z"), (2, 3)), z)
