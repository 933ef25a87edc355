"""ctypes binding of ``libmicmec_gb300.so`` (the C ABI in ``include/micmec_gb300.h``).

The library is built in-tree by :mod:`micmec_gb300.build`. There is no CPU
fallback: if the library or a CUDA device is missing, the first call raises.
"""

import ctypes
import os

__all__ = ["lib", "check", "MMError", "LIB_PATH", "MM_REC_LEN", "REC"]

# MICMEC_GB300_LIB selects another build of the library (e.g. one with different compile flags)
LIB_PATH = os.environ.get("MICMEC_GB300_LIB") or os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib",
                                                              "libmicmec_gb300.so")

MM_OK, MM_ERR_NAN, MM_ERR_ARG, MM_ERR_CUDA, MM_ERR_TIMEOUT = range(5)
MM_REC_LEN = 21
REC = {"epot": 0, "ekin": 1, "decons": 2, "vtens": slice(3, 12), "ktens": slice(12, 21)}

_lib = None

c_int = ctypes.c_int
c_int64 = ctypes.c_int64
c_uint64 = ctypes.c_uint64
c_double = ctypes.c_double
c_void_p = ctypes.c_void_p
P = ctypes.c_void_p  # raw pointers are passed as integers


class MMError(RuntimeError):
    """Error reported by the native library."""


def _declare(L):
    L.mm_create.argtypes = [c_int, c_int] + [P] * 5 + [c_int, c_int] + [P] * 6 + [c_int, c_int, ctypes.POINTER(c_void_p)]
    L.mm_destroy.argtypes = [c_void_p]
    L.mm_set_domain.argtypes = [c_void_p, P, P]
    L.mm_compute.argtypes = [c_void_p, P, P, P, P, P, c_void_p]
    L.mm_compute_host.argtypes = [c_void_p, P, P, P, P]
    L.mm_cell_results.argtypes = [c_void_p, P, P, c_void_p]
    L.mm_md_run.argtypes = [c_void_p, P, P, c_int, c_double, c_int, c_double, c_double, c_uint64, P, P, c_int64,
                            c_void_p]
    L.mm_md_begin.argtypes = [c_void_p, P, P, c_double, c_int, c_double, c_double, c_uint64, P, c_int64, c_void_p]
    L.mm_md_advance.argtypes = [c_void_p, c_int, P, c_int, c_void_p]
    L.mm_md_end.argtypes = [c_void_p, P, P, c_void_p]
    L.mm_md_step_host.argtypes = [c_void_p, P, P, P, P, c_double, c_int, c_double, c_double, c_uint64, c_int64]
    L.mm_md_time_kernels.argtypes = [c_void_p, c_int, P, ctypes.c_size_t, P, P, c_void_p]
    L.mm_set_params.argtypes = [c_void_p, P, P, P, P]
    L.mm_adjoint.argtypes = [c_void_p, P, P, P, P, P, P, P, P, c_void_p]
    L.mm_md_engine.argtypes = [c_void_p, P, P, c_int, c_double, c_int, c_double, c_double, c_int, c_double, c_int,
                               c_uint64, P, P, P, P, c_int64, c_void_p]
    L.mm_selftest_convert.argtypes = [P, P, P, P, c_int, c_void_p]
    L.mm_selftest_sym_exp.argtypes = [P, c_int, c_double, P, P, c_void_p]
    L.mm_build_topology.argtypes = [P, c_int, c_int, c_int, P, P, c_int, P, P, P, P, P, P, P, P, c_void_p]
    L.mm_last_error.restype = ctypes.c_char_p
    L.mm_version.restype = ctypes.c_char_p
    for name in ("mm_create", "mm_destroy", "mm_set_domain", "mm_compute", "mm_compute_host", "mm_cell_results",
                 "mm_md_run", "mm_md_begin", "mm_md_advance", "mm_md_end", "mm_md_step_host",
                 "mm_md_time_kernels", "mm_set_params", "mm_adjoint", "mm_md_engine", "mm_selftest_convert",
                 "mm_selftest_sym_exp", "mm_build_topology"):
        getattr(L, name).restype = c_int


def lib():
    """Load the library (once). Raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise MMError(
                "libmicmec_gb300.so is not built; run `python -c \"import __graft_entry__ as g; g.build()\"` "
                "or `python micmec_gb300/build.py`"
            )
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def check(status, what=""):
    """Map a status code to an exception: NaN -> ValueError (as the reference), others -> MMError."""
    if status == MM_OK:
        return
    msg = lib().mm_last_error().decode(errors="replace")
    if status == MM_ERR_NAN:
        raise ValueError("%s: not-a-number in energy, gradient or virial (%s)" % (what, msg))
    if status == MM_ERR_ARG:
        raise ValueError("%s: invalid argument (%s)" % (what, msg))
    if status == MM_ERR_TIMEOUT:
        raise MMError("%s: device wait timed out (%s)" % (what, msg))
    raise MMError("%s: CUDA error (%s)" % (what, msg))


def ptr(a):
    """Raw address of a torch tensor or NumPy array (or None -> NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data
