"""Python front end of the GPU CCSD(T) path (calls libgbcc through its C ABI).

Tensors are numpy arrays in the reference's index order (``T2[a, b, i, j]``,
``gamma[G, p, q]``); they are converted to the column-major buffers of the
ABI here.  Keyword names follow the oracle / reference YAML keys.
"""
import ctypes as C

import numpy as np

from . import capi
from .capi import fortran_flat, from_fortran_flat, ptr

__all__ = ["make_opts", "CcsdInput", "ccsd_solve", "ccsd_residual", "Solver",
           "triples", "coulomb_integrals", "energy", "ComplexInput",
           "ccsd_solve_complex", "ccsd_residual_complex", "triples_complex",
           "coulomb_integrals_pp", "coulomb_integrals_complex"]


def make_opts(mixer="LinearMixer", max_residua=4, mixing_ratio=1.0,
              max_iterations=16, energy_convergence=1e-6,
              amplitudes_convergence=1e-5, level_shift=0.0, distinguishable=0,
              ppl=1, slice_size=-1, slice_factor=None, precision="fp64",
              emu_slices=0, formulation="vertex", only_ppl=0, emu_min_flops=None,
              f64_split_blocks=None, emu_max_ksplit=None):
    o = capi.CcsdOpts()
    capi.load().gbcc_ccsd_opts_default(C.byref(o))
    o.mixer = {"LinearMixer": 0, "DiisMixer": 1}[mixer]
    o.max_residua = int(max_residua)
    o.mixing_ratio = float(mixing_ratio)
    o.max_iterations = int(max_iterations)
    o.energy_convergence = float(energy_convergence)
    o.amplitudes_convergence = float(amplitudes_convergence)
    o.level_shift = float(level_shift)
    o.distinguishable = int(distinguishable)
    o.ppl = int(ppl)
    o.integrals_slice_size = int(slice_size)
    o.integrals_slice_factor = -1.0 if slice_factor is None else float(slice_factor)
    o.precision = {"fp64": capi.PREC_FP64, "emu": capi.PREC_EMU}[precision]
    o.emu_slices = int(emu_slices)
    # "vertex": CcsdEnergyFromCoulombIntegrals; "stored":
    # CcsdEnergyFromCoulombIntegralsReference (resident Vabcd / Vabci)
    o.formulation = {"vertex": 0, "stored": 1}[formulation]
    o.only_ppl = int(only_ppl)
    # execution tuning (None: keep the context's setting)
    if emu_min_flops is not None:
        o.emu_min_flops = float(emu_min_flops)
    if f64_split_blocks is not None:
        o.f64_split_blocks = int(f64_split_blocks)
    if emu_max_ksplit is not None:
        o.emu_max_ksplit = int(emu_max_ksplit)
    return o


def _eigenenergies(eps_h, eps_p):
    eps_h = np.ascontiguousarray(eps_h, dtype=np.float64)
    eps_p = np.ascontiguousarray(eps_p, dtype=np.float64)
    if eps_h.ndim != 1 or eps_p.ndim != 1 or not eps_h.size or not eps_p.size:
        raise ValueError("eps_h and eps_p must be non-empty vectors")
    return eps_h, eps_p


def _flat(arr, shape, name):
    """Column-major copy of a real tensor after checking its shape.  The ABI
    takes bare pointers, so a wrong shape would be read past its end."""
    a = np.asarray(arr)
    if a.shape != tuple(shape):
        raise ValueError("%s has shape %s, expected %s" % (name, a.shape, tuple(shape)))
    if np.iscomplexobj(a):
        raise ValueError("%s must be real" % name)
    return fortran_flat(a)


def _vertex(gamma, No, Nv):
    """(column-major real vertex, its number of rows) for the real path.  The
    reference's real CCSD and (T) read a complex vertex Gamma[G, p, q] as
    Re.Re + Im.Im in every product of two vertex factors
    (CcsdEnergyFromCoulombIntegrals.cxx:80-115,162-169; CcsdPerturbativeTriples
    Complex.cxx:330-341), which is the real vertex [Re; Im] of 2 NG rows."""
    g = np.asarray(gamma)
    if g.ndim != 3 or g.shape[1:] != (No + Nv, No + Nv) or not g.shape[0]:
        raise ValueError("gamma has shape %s, expected (NG, %d, %d)"
                         % (g.shape, No + Nv, No + Nv))
    if np.iscomplexobj(g):
        if np.any(g.imag):
            return fortran_flat(np.concatenate([g.real, g.imag], axis=0)), 2 * g.shape[0]
        return fortran_flat(g.real), g.shape[0]
    return fortran_flat(g), g.shape[0]


_INTEGRAL_SHAPES = {"PPHH": "vvoo", "PHPH": "vovo", "HHHH": "oooo", "HHHP": "ooov",
                    "PPPP": "vvvv", "PPPH": "vvvo"}


def _shape(code, No, Nv):
    return tuple(No if c == "o" else Nv for c in code)


class CcsdInput:
    """Owns the column-major host buffers behind a ``gbcc_ccsd_in``.  The
    vertex may be None for the stored formulation when every integral it
    reads (PPHH, PHPH, HHHH, HHHP, PPPP, PPPH) is given."""

    def __init__(self, eps_h, eps_p, gamma, ints=None, initial=None, fock_hp=None):
        eps_h, eps_p = _eigenenergies(eps_h, eps_p)
        No, Nv = eps_h.size, eps_p.size
        if gamma is None:
            g, NG = None, 0
        else:
            g, NG = _vertex(gamma, No, Nv)
        self.No, self.Nv, self.NG = No, Nv, NG
        self._keep = [eps_h, eps_p, g]
        s = capi.CcsdIn()
        s.No, s.Nv, s.NG = self.No, self.Nv, self.NG
        s.eps_h, s.eps_p = ptr(eps_h), ptr(eps_p)
        s.gamma = ptr(g)
        ints = ints or {}
        for key, field in (("PPHH", "Vabij"), ("PHPH", "Vaibj"),
                           ("HHHH", "Vijkl"), ("HHHP", "Vijka"),
                           ("PPPP", "Vabcd"), ("PPPH", "Vabci")):
            if key in ints and ints[key] is not None:
                f = _flat(ints[key], _shape(_INTEGRAL_SHAPES[key], No, Nv), key)
                self._keep.append(f)
                setattr(s, field, ptr(f))
        if initial is not None:
            t1 = _flat(initial[0], (Nv, No), "initial T1")
            t2 = _flat(initial[1], (Nv, Nv, No, No), "initial T2")
            self._keep += [t1, t2]
            s.init_T1, s.init_T2 = ptr(t1), ptr(t2)
        if fock_hp is not None:  # HPFockMatrix f[i, a]
            f = _flat(fock_hp, (No, Nv), "fock_hp")
            self._keep.append(f)
            s.fock_hp = ptr(f)
        self.s = s


def ccsd_solve(ctx, eps_h, eps_p, gamma, ints=None, initial=None,
               want_amplitudes=True, pair_energy=False, fock_hp=None, **opts):
    inp = CcsdInput(eps_h, eps_p, gamma, ints, initial, fock_hp)
    o = make_opts(**opts)
    No, Nv = inp.No, inp.Nv
    out = capi.CcsdOut()
    t1 = np.zeros(Nv * No) if want_amplitudes else None
    t2 = np.zeros(Nv * Nv * No * No) if want_amplitudes else None
    pe = np.zeros(No * No) if pair_energy else None
    hist = np.zeros(max(o.max_iterations, 1))
    out.T1, out.T2, out.pair_energy, out.energy_history = ptr(t1), ptr(t2), ptr(pe), ptr(hist)
    st = ctx.check(ctx.lib.gbcc_ccsd_solve(ctx.h, C.byref(inp.s), C.byref(o),
                                           C.byref(out)),
                   allow=(capi.OK, capi.NOT_CONVERGED))
    r = {"energy": out.energy, "direct": out.direct, "exchange": out.exchange,
         "iterations": out.iterations, "converged": bool(out.converged),
         "status": st, "history": hist[:out.iterations].copy()}
    if want_amplitudes:
        r["T1"] = from_fortran_flat(t1, (Nv, No))
        r["T2"] = from_fortran_flat(t2, (Nv, Nv, No, No))
    if pair_energy:
        r["pair_energy"] = from_fortran_flat(pe, (No, No))
    return r


def ccsd_solve_batch(ctx, systems, want_amplitudes=False, **opts):
    """Solves several systems of one shape in lockstep
    (``gbcc_ccsd_solve_batch``): each contraction runs once for all of them.
    ``systems`` is a list of ``(eps_h, eps_p, gamma)`` or
    ``(eps_h, eps_p, gamma, initial)`` tuples.  Returns one result dict per
    system, as ``ccsd_solve`` gives it; a system that fails carries its error
    status in ``status`` instead of raising."""
    inps = [CcsdInput(*((sy[0], sy[1], sy[2]) + ((None, sy[3]) if len(sy) > 3 else ())))
            for sy in systems]
    n = len(inps)
    o = make_opts(**opts)
    outs = (capi.CcsdOut * n)()
    ins = (capi.CcsdIn * n)(*[i.s for i in inps])
    st = (C.c_int * n)()
    keep = []
    for z, inp in enumerate(inps):
        No, Nv = inp.No, inp.Nv
        hist = np.zeros(max(o.max_iterations, 1))
        t1 = np.zeros(Nv * No) if want_amplitudes else None
        t2 = np.zeros(Nv * Nv * No * No) if want_amplitudes else None
        outs[z].T1, outs[z].T2, outs[z].energy_history = ptr(t1), ptr(t2), ptr(hist)
        keep.append((hist, t1, t2))
    ctx.check(ctx.lib.gbcc_ccsd_solve_batch(ctx.h, n, ins, C.byref(o), outs, st))
    res = []
    for z, inp in enumerate(inps):
        out = outs[z]
        hist, t1, t2 = keep[z]
        r = {"energy": out.energy, "direct": out.direct, "exchange": out.exchange,
             "iterations": out.iterations, "converged": bool(out.converged),
             "status": st[z], "history": hist[:out.iterations].copy()}
        if want_amplitudes:
            r["T1"] = from_fortran_flat(t1, (inp.Nv, inp.No))
            r["T2"] = from_fortran_flat(t2, (inp.Nv, inp.Nv, inp.No, inp.No))
        res.append(r)
    return res


def ccsd_residual(ctx, it, T1, T2, eps_h, eps_p, gamma, ints=None,
                  initial=None, **opts):
    inp = CcsdInput(eps_h, eps_p, gamma, ints, initial)
    o = make_opts(**opts)
    No, Nv = inp.No, inp.Nv
    t1, t2 = fortran_flat(T1), fortran_flat(T2)
    r1 = np.zeros(Nv * No)
    r2 = np.zeros(Nv * Nv * No * No)
    ctx.check(ctx.lib.gbcc_ccsd_residual(ctx.h, C.byref(inp.s), C.byref(o),
                                         int(it), ptr(t1), ptr(t2), ptr(r1),
                                         ptr(r2)))
    return (from_fortran_flat(r1, (Nv, No)),
            from_fortran_flat(r2, (Nv, Nv, No, No)))


class Solver:
    """Device-resident solver: inputs uploaded once, iterations on demand."""

    def __init__(self, ctx, eps_h, eps_p, gamma, ints=None, initial=None,
                 fock_hp=None, **opts):
        self.ctx = ctx
        self.inp = CcsdInput(eps_h, eps_p, gamma, ints, initial, fock_hp)
        self.opts = make_opts(**opts)
        h = C.c_void_p()
        ctx.check(ctx.lib.gbcc_ccsd_setup(ctx.h, C.byref(self.inp.s),
                                          C.byref(self.opts), C.byref(h)))
        self.h = h

    def step(self, n=1):
        e = C.c_double()
        conv = C.c_int()
        self.ctx.check(self.ctx.lib.gbcc_ccsd_step(self.h, int(n), C.byref(e),
                                                   C.byref(conv)))
        return e.value, bool(conv.value)

    def restart(self):
        """Back to the starting amplitudes with no iterations done; the
        resident inputs and captured iteration graphs are kept."""
        self.ctx.check(self.ctx.lib.gbcc_ccsd_restart(self.h))

    def result(self, amplitudes=True):
        """Energy, iteration count, the energy of every iteration since the
        start (or the last restart) and, optionally, the amplitudes."""
        No, Nv = self.inp.No, self.inp.Nv
        out = capi.CcsdOut()
        t1 = np.zeros(Nv * No) if amplitudes else None
        t2 = np.zeros(Nv * Nv * No * No) if amplitudes else None
        hist = np.zeros(max(self.opts.max_iterations, 1))
        out.T1, out.T2, out.energy_history = ptr(t1), ptr(t2), ptr(hist)
        self.ctx.check(self.ctx.lib.gbcc_ccsd_result(self.h, C.byref(out)))
        r = {"energy": out.energy, "iterations": out.iterations,
             "converged": bool(out.converged),
             "history": hist[:out.iterations].copy()}
        if amplitudes:
            r["T1"] = from_fortran_flat(t1, (Nv, No))
            r["T2"] = from_fortran_flat(t2, (Nv, Nv, No, No))
        return r

    def triples(self, precision="fp64"):
        et, etot = C.c_double(), C.c_double()
        p = {"fp64": capi.PREC_FP64, "emu": capi.PREC_EMU}[precision]
        self.ctx.check(self.ctx.lib.gbcc_triples_from_solver(
            self.h, p, C.byref(etot), C.byref(et)))
        return et.value, etot.value

    def close(self):
        if getattr(self, "h", None):
            self.ctx.lib.gbcc_ccsd_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def triples(ctx, eps_h, eps_p, gamma, T1, T2, e_ccsd=0.0, Vabij=None,
            Vijka=None, precision="fp64"):
    """Returns (E_(T), E_CCSD + E_(T))."""
    eps_h, eps_p = _eigenenergies(eps_h, eps_p)
    No, Nv = eps_h.size, eps_p.size
    g, NG = _vertex(gamma, No, Nv)
    s = capi.TriplesIn()
    s.No, s.Nv, s.NG = No, Nv, NG
    keep = [eps_h, eps_p, g]
    s.eps_h, s.eps_p = ptr(eps_h), ptr(eps_p)
    s.gamma = ptr(g)
    for name, arr, shape in (("T1", T1, (Nv, No)), ("T2", T2, (Nv, Nv, No, No)),
                             ("Vabij", Vabij, (Nv, Nv, No, No)),
                             ("Vijka", Vijka, (No, No, No, Nv))):
        if arr is not None:
            f = _flat(arr, shape, name)
            keep.append(f)
            setattr(s, name, ptr(f))
    s.e_ccsd = float(e_ccsd)
    et, etot = C.c_double(), C.c_double()
    p = {"fp64": capi.PREC_FP64, "emu": capi.PREC_EMU}[precision]
    ctx.check(ctx.lib.gbcc_triples(ctx.h, C.byref(s), p, C.byref(etot),
                                   C.byref(et)))
    del keep
    return et.value, etot.value


def coulomb_integrals(ctx, gamma, No):
    NG, Np = np.shape(gamma)[0], np.shape(gamma)[1]
    Nv = Np - No
    if not 0 < No < Np:
        raise ValueError("No must lie in 1..Np-1")
    g, NG = _vertex(gamma, No, Nv)
    vabij = np.zeros(Nv * Nv * No * No)
    vaibj = np.zeros(Nv * Nv * No * No)
    vijkl = np.zeros(No ** 4)
    vijka = np.zeros(No ** 3 * Nv)
    vijab = np.zeros(Nv * Nv * No * No)
    ctx.check(ctx.lib.gbcc_coulomb_integrals(ctx.h, No, Nv, NG, ptr(g),
                                             ptr(vabij), ptr(vaibj),
                                             ptr(vijkl), ptr(vijka),
                                             ptr(vijab)))
    return {"PPHH": from_fortran_flat(vabij, (Nv, Nv, No, No)),
            "PHPH": from_fortran_flat(vaibj, (Nv, No, Nv, No)),
            "HHHH": from_fortran_flat(vijkl, (No, No, No, No)),
            "HHHP": from_fortran_flat(vijka, (No, No, No, Nv)),
            "HHPP": from_fortran_flat(vijab, (No, No, Nv, Nv))}


def coulomb_integrals_pp(ctx, gamma, No):
    """PPPP (Vabcd) and PPPH (Vabci) integrals of the stored formulation."""
    NG, Np = np.shape(gamma)[0], np.shape(gamma)[1]
    Nv = Np - No
    if not 0 < No < Np:
        raise ValueError("No must lie in 1..Np-1")
    g, NG = _vertex(gamma, No, Nv)
    vabcd = np.zeros(Nv ** 4)
    vabci = np.zeros(Nv ** 3 * No)
    ctx.check(ctx.lib.gbcc_coulomb_integrals_pp(ctx.h, No, Nv, NG, ptr(g), ptr(vabcd),
                                                ptr(vabci)))
    return {"PPPP": from_fortran_flat(vabcd, (Nv, Nv, Nv, Nv)),
            "PPPH": from_fortran_flat(vabci, (Nv, Nv, Nv, No))}


# ------------------------------------------------------------- complex branch
def complex_flat(arr, shape, name):
    """Interleaved (re, im) column-major copy of a complex tensor, after
    checking its shape: the layout of CTF's complex<double> tensors."""
    a = np.asarray(arr)
    if a.shape != tuple(shape):
        raise ValueError("%s has shape %s, expected %s" % (name, a.shape, tuple(shape)))
    z = np.ascontiguousarray(np.asarray(a, dtype=np.complex128).transpose(
        tuple(range(a.ndim - 1, -1, -1)))).ravel()
    return z.view(np.float64)


def from_complex_flat(flat, shape):
    z = np.asarray(flat).view(np.complex128)
    return z.reshape(tuple(reversed(shape))).transpose(
        tuple(range(len(shape) - 1, -1, -1)))


class ComplexInput:
    """Owns the host buffers behind a ``gbcc_ccsd_complex_in``."""

    def __init__(self, eps_h, eps_p, gamma, initial=None, fock_hp=None):
        eps_h, eps_p = _eigenenergies(eps_h, eps_p)
        No, Nv = eps_h.size, eps_p.size
        g = np.asarray(gamma)
        if g.ndim != 3 or not g.shape[0]:
            raise ValueError("gamma must be [NG, Np, Np]")
        NG = g.shape[0]
        self.No, self.Nv, self.NG = No, Nv, NG
        gf = complex_flat(g, (NG, No + Nv, No + Nv), "gamma")
        self._keep = [eps_h, eps_p, gf]
        s = capi.ComplexIn()
        s.No, s.Nv, s.NG = No, Nv, NG
        s.eps_h, s.eps_p, s.gamma = ptr(eps_h), ptr(eps_p), ptr(gf)
        if initial is not None:
            t1 = complex_flat(initial[0], (Nv, No), "initial T1")
            t2 = complex_flat(initial[1], (Nv, Nv, No, No), "initial T2")
            self._keep += [t1, t2]
            s.init_T1, s.init_T2 = ptr(t1), ptr(t2)
        if fock_hp is not None:  # HPFockMatrix f[i, a]
            f = complex_flat(fock_hp, (No, Nv), "fock_hp")
            self._keep.append(f)
            s.fock_hp = ptr(f)
        self.s = s


def ccsd_solve_complex(ctx, eps_h, eps_p, gamma, initial=None, fock_hp=None,
                       pair_energy=False, **opts):
    """Complex CCSD (linear mixer).  Returns complex energies, the complex
    per-iteration history, the complex amplitudes and, on request, the
    complex pair energies."""
    inp = ComplexInput(eps_h, eps_p, gamma, initial, fock_hp)
    o = make_opts(**opts)
    No, Nv = inp.No, inp.Nv
    out = capi.ComplexOut()
    t1 = np.zeros(2 * Nv * No)
    t2 = np.zeros(2 * Nv * Nv * No * No)
    hist = np.zeros(2 * max(o.max_iterations, 1))
    pe = np.zeros(2 * No * No) if pair_energy else None
    out.T1, out.T2, out.energy_history = ptr(t1), ptr(t2), ptr(hist)
    out.pair_energy = ptr(pe)
    st = ctx.check(ctx.lib.gbcc_ccsd_solve_complex(ctx.h, C.byref(inp.s), C.byref(o),
                                                   C.byref(out)),
                   allow=(capi.OK, capi.NOT_CONVERGED))
    n = out.iterations
    return {"energy": complex(out.energy[0], out.energy[1]),
            "direct": complex(out.direct[0], out.direct[1]),
            "exchange": complex(out.exchange[0], out.exchange[1]),
            "iterations": n, "converged": bool(out.converged), "status": st,
            "history": hist[:2 * n].view(np.complex128).copy(),
            "T1": from_complex_flat(t1, (Nv, No)),
            "T2": from_complex_flat(t2, (Nv, Nv, No, No)),
            "pair_energy": None if pe is None else from_complex_flat(pe, (No, No))}


def ccsd_residual_complex(ctx, it, T1, T2, eps_h, eps_p, gamma,
                          initial_doubles=False, **opts):
    """One complex getResiduum call; ``initial_doubles`` selects the
    reference's behaviour when initialDoublesAmplitudes is given (no MP2
    start at it = 0)."""
    inp = ComplexInput(eps_h, eps_p, gamma)
    o = make_opts(**opts)
    No, Nv = inp.No, inp.Nv
    t1 = complex_flat(T1, (Nv, No), "T1")
    t2 = complex_flat(T2, (Nv, Nv, No, No), "T2")
    if initial_doubles:
        inp.s.init_T2 = ptr(t2)
    r1 = np.zeros(2 * Nv * No)
    r2 = np.zeros(2 * Nv * Nv * No * No)
    ctx.check(ctx.lib.gbcc_ccsd_residual_complex(ctx.h, C.byref(inp.s), C.byref(o),
                                                 int(it), ptr(t1), ptr(t2), ptr(r1),
                                                 ptr(r2)))
    return from_complex_flat(r1, (Nv, No)), from_complex_flat(r2, (Nv, Nv, No, No))


def triples_complex(ctx, eps_h, eps_p, gamma, T1, T2, e_ccsd=0.0, precision="fp64"):
    """CcsdPerturbativeTriplesComplex: returns (complex E_(T), e_ccsd + Re E_(T))."""
    eps_h, eps_p = _eigenenergies(eps_h, eps_p)
    No, Nv = eps_h.size, eps_p.size
    g = np.asarray(gamma)
    if g.ndim != 3 or not g.shape[0]:
        raise ValueError("gamma must be [NG, Np, Np]")
    NG = g.shape[0]
    keep = [eps_h, eps_p, complex_flat(g, (NG, No + Nv, No + Nv), "gamma"),
            complex_flat(T1, (Nv, No), "T1"), complex_flat(T2, (Nv, Nv, No, No), "T2")]
    s = capi.TriplesComplexIn()
    s.No, s.Nv, s.NG = No, Nv, NG
    s.eps_h, s.eps_p, s.gamma, s.T1, s.T2 = [ptr(a) for a in keep]
    s.e_ccsd = float(e_ccsd)
    et = np.zeros(2)
    etot = C.c_double()
    p = {"fp64": capi.PREC_FP64, "emu": capi.PREC_EMU}[precision]
    ctx.check(ctx.lib.gbcc_triples_complex(ctx.h, C.byref(s), p, C.byref(etot), ptr(et)))
    del keep
    return complex(et[0], et[1]), etot.value


def coulomb_integrals_complex(ctx, gamma, No):
    """Complex integrals of CoulombIntegralsFromVertex with complex: 1 (PPHH,
    PHHP, HHPP, PHPH, HHHH, HHHP, PHHH) from a complex vertex."""
    g = np.asarray(gamma)
    NG, Np = g.shape[0], g.shape[1]
    Nv = Np - No
    if g.ndim != 3 or not 0 < No < Np:
        raise ValueError("gamma must be [NG, Np, Np] with 0 < No < Np")
    gf = complex_flat(g, (NG, Np, Np), "gamma")
    shapes = {"PPHH": (Nv, Nv, No, No), "PHHP": (Nv, No, No, Nv), "HHPP": (No, No, Nv, Nv),
              "PHPH": (Nv, No, Nv, No), "HHHH": (No, No, No, No), "HHHP": (No, No, No, Nv),
              "PHHH": (Nv, No, No, No)}
    bufs = {k: np.zeros(2 * int(np.prod(v))) for k, v in shapes.items()}
    ctx.check(ctx.lib.gbcc_coulomb_integrals_complex(
        ctx.h, No, Nv, NG, ptr(gf), *[ptr(bufs[k]) for k in shapes]))
    return {k: from_complex_flat(bufs[k], shapes[k]) for k in shapes}
