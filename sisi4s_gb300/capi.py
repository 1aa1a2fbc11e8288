"""ctypes binding of libgbcc.so (include/gbcc.h).

Loads the in-tree library built by ``sisi4s_gb300.build``.  There is no CPU
fallback: if the library or a CUDA device is missing, the calls raise.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libgbcc.so")

OK, NOT_CONVERGED, DIIS_SINGULAR, DIVERGED, OOM, BAD_ARG, CUDA_ERROR, \
    TIMEOUT, COMPLEX_UNSUPPORTED, NO_DEVICE = range(10)
PREC_FP64, PREC_EMU = 0, 1
FAULT_NONE, FAULT_DIIS_SINGULAR, FAULT_NAN, FAULT_OOM, FAULT_DEVICE_WAIT = range(5)

_dp = C.POINTER(C.c_double)


class CcsdOpts(C.Structure):
    _fields_ = [("mixer", C.c_int), ("max_residua", C.c_int),
                ("mixing_ratio", C.c_double), ("max_iterations", C.c_int),
                ("energy_convergence", C.c_double),
                ("amplitudes_convergence", C.c_double),
                ("level_shift", C.c_double), ("distinguishable", C.c_int),
                ("ppl", C.c_int), ("integrals_slice_size", C.c_int),
                ("integrals_slice_factor", C.c_double),
                ("precision", C.c_int), ("emu_slices", C.c_int),
                ("formulation", C.c_int), ("only_ppl", C.c_int),
                ("emu_min_flops", C.c_double), ("f64_split_blocks", C.c_int),
                ("emu_max_ksplit", C.c_int)]


class CcsdIn(C.Structure):
    _fields_ = [("No", C.c_int), ("Nv", C.c_int), ("NG", C.c_int),
                ("eps_h", _dp), ("eps_p", _dp), ("gamma", _dp),
                ("gamma_imag", _dp), ("Vabij", _dp), ("Vaibj", _dp),
                ("Vijkl", _dp), ("Vijka", _dp), ("init_T1", _dp),
                ("init_T2", _dp), ("fock_hp", _dp), ("Vabcd", _dp),
                ("Vabci", _dp)]


class CcsdOut(C.Structure):
    _fields_ = [("energy", C.c_double), ("direct", C.c_double),
                ("exchange", C.c_double), ("iterations", C.c_int),
                ("converged", C.c_int), ("T1", _dp), ("T2", _dp),
                ("pair_energy", _dp), ("energy_history", _dp)]


class ComplexIn(C.Structure):
    _fields_ = [("No", C.c_int), ("Nv", C.c_int), ("NG", C.c_int),
                ("eps_h", _dp), ("eps_p", _dp), ("gamma", _dp),
                ("init_T1", _dp), ("init_T2", _dp), ("fock_hp", _dp)]


class ComplexOut(C.Structure):
    _fields_ = [("energy", C.c_double * 2), ("direct", C.c_double * 2),
                ("exchange", C.c_double * 2), ("iterations", C.c_int),
                ("converged", C.c_int), ("T1", _dp), ("T2", _dp),
                ("energy_history", _dp), ("pair_energy", _dp)]


class TriplesComplexIn(C.Structure):
    _fields_ = [("No", C.c_int), ("Nv", C.c_int), ("NG", C.c_int),
                ("eps_h", _dp), ("eps_p", _dp), ("gamma", _dp),
                ("T1", _dp), ("T2", _dp), ("e_ccsd", C.c_double)]


class TriplesIn(C.Structure):
    _fields_ = [("No", C.c_int), ("Nv", C.c_int), ("NG", C.c_int),
                ("eps_h", _dp), ("eps_p", _dp), ("gamma", _dp),
                ("gamma_imag", _dp), ("Vabij", _dp), ("Vijka", _dp),
                ("T1", _dp), ("T2", _dp), ("e_ccsd", C.c_double)]


_SIGS = {
    "gbcc_abi_version": (C.c_int, []),
    "gbcc_status_string": (C.c_char_p, [C.c_int]),
    "gbcc_ctx_create": (C.c_int, [C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]),
    "gbcc_ctx_destroy": (None, [C.c_void_p]),
    "gbcc_last_error": (C.c_char_p, [C.c_void_p]),
    "gbcc_ctx_kernel_launches": (C.c_uint64, [C.c_void_p]),
    "gbcc_ctx_flops": (C.c_double, [C.c_void_p]),
    "gbcc_ctx_stream": (C.c_void_p, [C.c_void_p]),
    "gbcc_device_pool_high_water": (C.c_int, [C.c_int, C.c_int, C.POINTER(C.c_int64)]),
    "gbcc_ctx_set_emulation": (C.c_int, [C.c_void_p, C.c_int, C.c_double]),
    "gbcc_ctx_set_triples_batch": (C.c_int, [C.c_void_p, C.c_int]),
    "gbcc_ctx_set_splits": (C.c_int, [C.c_void_p, C.c_int, C.c_int]),
    "gbcc_ctx_set_operand_cache": (C.c_int, [C.c_void_p, C.c_int]),
    "gbcc_ctx_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "gbcc_ctx_set_graphs": (C.c_int, [C.c_void_p, C.c_int]),
    "gbcc_ctx_gemm_stats": (C.c_int, [C.c_void_p, _dp, C.POINTER(C.c_int64),
                                      _dp, _dp]),
    "gbcc_ctx_inject_fault": (C.c_int, [C.c_void_p, C.c_int]),
    "gbcc_ctx_gemm_records": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), _dp,
                                        C.c_int64, C.POINTER(C.c_int64)]),
    "gbcc_ccsd_opts_default": (None, [C.POINTER(CcsdOpts)]),
    "gbcc_ccsd_solve": (C.c_int, [C.c_void_p, C.POINTER(CcsdIn),
                                  C.POINTER(CcsdOpts), C.POINTER(CcsdOut)]),
    "gbcc_ccsd_solve_batch": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(CcsdIn),
                                        C.POINTER(CcsdOpts), C.POINTER(CcsdOut),
                                        C.POINTER(C.c_int)]),
    "gbcc_ccsd_setup": (C.c_int, [C.c_void_p, C.POINTER(CcsdIn),
                                  C.POINTER(CcsdOpts), C.POINTER(C.c_void_p)]),
    "gbcc_ccsd_step": (C.c_int, [C.c_void_p, C.c_int, _dp,
                                 C.POINTER(C.c_int)]),
    "gbcc_ccsd_result": (C.c_int, [C.c_void_p, C.POINTER(CcsdOut)]),
    "gbcc_ccsd_device_amplitudes": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p),
                                              C.POINTER(C.c_void_p)]),
    "gbcc_ccsd_destroy": (None, [C.c_void_p]),
    "gbcc_ccsd_restart": (C.c_int, [C.c_void_p]),
    "gbcc_ccsd_residual": (C.c_int, [C.c_void_p, C.POINTER(CcsdIn),
                                     C.POINTER(CcsdOpts), C.c_int, _dp, _dp,
                                     _dp, _dp]),
    "gbcc_ccsd_solve_complex": (C.c_int, [C.c_void_p, C.POINTER(ComplexIn),
                                          C.POINTER(CcsdOpts), C.POINTER(ComplexOut)]),
    "gbcc_ccsd_residual_complex": (C.c_int, [C.c_void_p, C.POINTER(ComplexIn),
                                             C.POINTER(CcsdOpts), C.c_int, _dp, _dp,
                                             _dp, _dp]),
    "gbcc_triples": (C.c_int, [C.c_void_p, C.POINTER(TriplesIn), C.c_int,
                               _dp, _dp]),
    "gbcc_triples_complex": (C.c_int, [C.c_void_p, C.POINTER(TriplesComplexIn), C.c_int,
                                       _dp, _dp]),
    "gbcc_triples_from_solver": (C.c_int, [C.c_void_p, C.c_int, _dp, _dp]),
    "gbcc_coulomb_integrals": (C.c_int, [C.c_void_p, C.c_int, C.c_int,
                                         C.c_int, _dp, _dp, _dp, _dp, _dp,
                                         _dp]),
    "gbcc_coulomb_integrals_pp": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int,
                                            _dp, _dp, _dp]),
    "gbcc_coulomb_integrals_complex": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int,
                                                 _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]),
    "gbcc_dgemm": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int64,
                             C.c_int64, C.c_int64, C.c_double, C.c_void_p,
                             C.c_int64, C.c_void_p, C.c_int64, C.c_double,
                             C.c_void_p, C.c_int64, C.c_int]),
    "gbcc_dgemm_emu_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_int,
                                         C.c_int64, C.c_int64, C.c_int64,
                                         C.c_double, C.c_void_p, C.c_int64,
                                         C.c_void_p, C.c_int64, C.c_double,
                                         C.c_void_p, C.c_int64]),
    "gbcc_energy": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p,
                              C.c_void_p, C.c_void_p, _dp, _dp]),
}

_lib = None


def load(path=LIB_PATH):
    """Load libgbcc.so (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build
        build.build()
    lib = C.CDLL(path)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class GbccError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s: %s" % (status_string(status), msg))
        self.status = status


def status_string(s):
    return load().gbcc_status_string(s).decode()


def ptr(a):
    """double* of a C-contiguous float64 array (None -> NULL)."""
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_dp)


def fortran_flat(a):
    """Column-major (first index fastest) flat copy of a numpy tensor."""
    return np.ascontiguousarray(np.asarray(a, dtype=np.float64).transpose(
        tuple(range(a.ndim - 1, -1, -1)))).ravel()


def from_fortran_flat(flat, shape):
    return np.asarray(flat).reshape(tuple(reversed(shape))).transpose(
        tuple(range(len(shape) - 1, -1, -1)))


class Context:
    """A device context (one stream)."""

    def __init__(self, device=0, stream=None):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.gbcc_ctx_create(device, stream, C.byref(h))
        if st != OK:
            raise GbccError(st, self.lib.gbcc_last_error(None).decode())
        self.h = h
        self.device = device

    def check(self, st, allow=(OK,)):
        if st not in allow:
            raise GbccError(st, self.lib.gbcc_last_error(self.h).decode())
        return st

    def set_emulation(self, slices=6, min_flops=1e7):
        self.check(self.lib.gbcc_ctx_set_emulation(self.h, int(slices),
                                                   float(min_flops)))

    def set_triples_batch(self, max_images=0):
        """(T) batch bound in distinct triple images (0: automatic)."""
        self.check(self.lib.gbcc_ctx_set_triples_batch(self.h, int(max_images)))

    def set_splits(self, f64_blocks_per_sm=3, emu_max_ksplit=64):
        """K-split policies of the FP64 and emulated GEMMs (defaults shown)."""
        self.check(self.lib.gbcc_ctx_set_splits(self.h, int(f64_blocks_per_sm),
                                                int(emu_max_ksplit)))

    def set_operand_cache(self, enable=True):
        """Reuse of the digit panels of a solver's constant operands."""
        self.check(self.lib.gbcc_ctx_set_operand_cache(self.h, int(bool(enable))))

    def set_graphs(self, enable=True):
        self.check(self.lib.gbcc_ctx_set_graphs(self.h, 1 if enable else 0))

    def profile(self, enable=True):
        self.check(self.lib.gbcc_ctx_profile(self.h, 1 if enable else 0))

    def gemm_stats(self):
        ms, n = C.c_double(), C.c_int64()
        tc, f64 = C.c_double(), C.c_double()
        self.check(self.lib.gbcc_ctx_gemm_stats(self.h, C.byref(ms), C.byref(n),
                                                C.byref(tc), C.byref(f64)))
        return {"ms": ms.value, "launches": n.value, "tc_flops": tc.value,
                "fp64_flops": f64.value}

    def inject_fault(self, kind):
        """Make the next event of ``kind`` (FAULT_*) fail once (tests)."""
        self.check(self.lib.gbcc_ctx_inject_fault(self.h, int(kind)))

    def gemm_records(self, cap=1 << 16):
        """[(M, N, K, ms)] of the profiled GEMM launches since the last call."""
        mnk = np.zeros(3 * cap, dtype=np.int64)
        ms = np.zeros(cap)
        n = C.c_int64()
        self.check(self.lib.gbcc_ctx_gemm_records(
            self.h, mnk.ctypes.data_as(C.POINTER(C.c_int64)), ptr(ms), cap, C.byref(n)))
        return [(int(mnk[3 * i]), int(mnk[3 * i + 1]), int(mnk[3 * i + 2]), float(ms[i]))
                for i in range(n.value)]

    def pool_high_water(self, reset=False):
        """Peak bytes held by the library's device allocations on this
        context's device since the last reset (reset=True starts over)."""
        v = C.c_int64()
        self.check(self.lib.gbcc_device_pool_high_water(self.device, int(reset),
                                                        C.byref(v)))
        return v.value

    @property
    def launches(self):
        return int(self.lib.gbcc_ctx_kernel_launches(self.h))

    @property
    def flops(self):
        return float(self.lib.gbcc_ctx_flops(self.h))

    @property
    def stream(self):
        return self.lib.gbcc_ctx_stream(self.h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.gbcc_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
