"""Host-side argument checks of the Python front end (no GPU).

The C ABI takes bare pointers and sizes, so the front end refuses arrays of
the wrong shape before anything reaches the library, and hands a complex
vertex's imaginary part to the library (which refuses it unless it is zero)
instead of dropping it in a float64 cast.
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
    assert inp.gamma_imag is None and not inp.s.gamma_imag
    assert (inp.No, inp.Nv, inp.NG) == (No, Nv, NG)


def test_complex_vertex_keeps_its_imaginary_part(system):
    g = system.gamma.astype(np.complex128)
    g[1, 2, 3] += 1e-3j
    inp = gpu.CcsdInput(system.eps_h, system.eps_p, g)
    assert inp.s.gamma_imag
    # column-major: element (G, p, q) sits at G + p*NG + q*NG*Np
    Np = No + Nv
    assert inp.gamma_imag[1 + 2 * NG + 3 * NG * Np] == 1e-3
    assert np.count_nonzero(inp.gamma_imag) == 1


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
