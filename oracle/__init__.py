"""CPU oracle (TEST INFRASTRUCTURE ONLY): ctypes access to oracle/liboracle.so,
the C restatement of the reference's sigma / Davidson / RQ-CG path, and to
oracle/_ref/libdoci_ref.so, the reference itself compiled from its sources
(present only where the reference checkout was available at build time).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use this
module, to check results and to time the CPU path.  The product (doci_gb300/)
never imports it.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
REF_LIB_PATH = os.path.join(HERE, "_ref", "libdoci_ref.so")
REF_EXE_PATH = os.path.join(HERE, "_ref", "doci_ref")
REF_EXE_PLAIN_PATH = os.path.join(HERE, "_ref", "doci_ref_plain")
_pd = C.POINTER(C.c_double)
_pu64 = C.POINTER(C.c_uint64)


class OrcHam(C.Structure):
    _fields_ = [("L", C.c_uint), ("N", C.c_uint), ("D", C.c_uint64), ("core", C.c_double),
                ("one", _pd), ("two", _pd), ("K", _pd), ("diag", _pd)]


_O = None


def build(ref: bool = False) -> None:
    subprocess.run(["make", "-s", "-C", HERE, "liboracle.so"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def lib() -> C.CDLL:
    global _O
    if _O is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.orc_ham_create.argtypes = [C.c_char_p, C.c_int, C.POINTER(C.POINTER(OrcHam))]
        L.orc_ham_destroy.argtypes = [C.POINTER(OrcHam)]
        L.orc_matvec.argtypes = [C.POINTER(OrcHam), _pd, _pd, C.c_int]
        L.orc_matvec_gather_rows.argtypes = [C.POINTER(OrcHam), _pd, _pd, _pu64, _pu64, C.c_int, _pd, C.c_int]
        L.orc_diagonal_range.argtypes = [C.POINTER(OrcHam), C.c_uint64, C.c_uint64, _pd]
        L.orc_bitstrings.argtypes = [C.c_uint, C.c_uint, C.POINTER(C.c_uint32)]
        L.orc_rank.argtypes = [C.c_uint32, C.c_uint, C.c_uint]
        L.orc_rank.restype = C.c_uint64
        L.orc_unrank.argtypes = [C.c_uint64, C.c_uint, C.c_uint]
        L.orc_unrank.restype = C.c_uint32
        L.orc_binom.argtypes = [C.c_uint, C.c_uint]
        L.orc_binom.restype = C.c_uint64
        L.orc_jacobi_eig.argtypes = [C.c_int, _pd, C.c_int, _pd, _pd]
        L.orc_davidson.argtypes = [C.POINTER(OrcHam), _pd, _pd, C.c_int, C.c_int, C.c_double, C.c_int,
                                   C.POINTER(C.c_int), _pd]
        L.orc_ray_q.argtypes = [C.POINTER(OrcHam), _pd, _pd, C.c_double, C.c_int, C.c_int, C.POINTER(C.c_int), _pd]
        L.orc_hf_index.argtypes = [C.POINTER(OrcHam)]
        L.orc_hf_index.restype = C.c_uint64
        L.orc_read_fcidump.argtypes = [C.c_char_p, C.POINTER(C.c_uint), C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                       _pd, C.POINTER(_pd), C.POINTER(_pd), C.POINTER(C.c_int)]
        _O = L
    return _O


def _p(a):
    return a.ctypes.data_as(_pd)


class Ham:
    """Oracle Hamiltonian (doci.c:69-134 restated)."""

    def __init__(self, fcidump: str, keep_diag: bool = True):
        self._h = C.POINTER(OrcHam)()
        st = lib().orc_ham_create(os.fsencode(fcidump), int(keep_diag), C.byref(self._h))
        if st:
            raise RuntimeError(f"orc_ham_create({fcidump}) failed with status {st}")
        c = self._h.contents
        self.L, self.N, self.D, self.core = c.L, c.N, c.D, c.core

    def close(self):
        if self._h:
            lib().orc_ham_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def diag(self) -> np.ndarray:
        return np.ctypeslib.as_array(self._h.contents.diag, (self.D,)).copy()

    @property
    def K(self) -> np.ndarray:
        return np.ctypeslib.as_array(self._h.contents.K, (self.L * self.L,)).reshape(self.L, self.L).copy()

    def matvec(self, x: np.ndarray, nthreads: int = 0) -> np.ndarray:
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        lib().orc_matvec(self._h, _p(x), _p(y), nthreads)
        return y

    def gather_rows(self, x, first, length, diag_rows, nthreads: int = 0) -> np.ndarray:
        first = np.ascontiguousarray(first, dtype=np.uint64)
        length = np.ascontiguousarray(length, dtype=np.uint64)
        diag_rows = np.ascontiguousarray(diag_rows, dtype=np.float64)
        y = np.empty(int(length.sum()), dtype=np.float64)
        lib().orc_matvec_gather_rows(self._h, _p(x), _p(diag_rows), first.ctypes.data_as(_pu64),
                                     length.ctypes.data_as(_pu64), len(first), _p(y), nthreads)
        return y

    def diagonal_range(self, first: int, count: int) -> np.ndarray:
        out = np.empty(count, dtype=np.float64)
        lib().orc_diagonal_range(self._h, first, count, _p(out))
        return out

    def davidson(self, x0=None, max_vectors=30, keep=2, tol=1e-8, max_its=200):
        x = np.zeros(self.D) if x0 is None else np.array(x0, dtype=np.float64)
        if x0 is None:
            x[lib().orc_hf_index(self._h)] = 1.0
        e = C.c_double()
        its = C.c_int()
        trace = np.zeros(2 * max_its + 2)
        rc = lib().orc_davidson(self._h, _p(x), C.byref(e), max_vectors, keep, tol, max_its, C.byref(its), _p(trace))
        n = min(its.value, max_its)
        return {"energy": e.value, "iterations": its.value, "return_code": rc,
                "trace": trace[:2 * n].reshape(n, 2)}, x

    def ray_q(self, x0=None, tol=1e-8, max_its=200, precond=False):
        x = np.zeros(self.D) if x0 is None else np.array(x0, dtype=np.float64)
        if x0 is None:
            x[lib().orc_hf_index(self._h)] = 1.0
        e = C.c_double()
        its = C.c_int()
        trace = np.zeros(2 * max_its + 2)
        rc = lib().orc_ray_q(self._h, _p(x), C.byref(e), tol, max_its, int(precond), C.byref(its), _p(trace))
        n = min(its.value, max_its)
        return {"energy": e.value, "iterations": its.value, "return_code": rc,
                "trace": trace[:2 * n].reshape(n, 2)}, x


def bitstrings(L: int, N: int) -> np.ndarray:
    D = lib().orc_binom(L, N)
    out = np.empty(D, dtype=np.uint32)
    lib().orc_bitstrings(N, L, out.ctypes.data_as(C.POINTER(C.c_uint32)))
    return out


def jacobi_eig(A: np.ndarray):
    A = np.asfortranarray(A, dtype=np.float64)
    n = A.shape[0]
    w = np.empty(n)
    V = np.empty((n, n), order="F")
    lib().orc_jacobi_eig(n, A.ctypes.data_as(_pd), n, _p(w), V.ctypes.data_as(_pd))
    return w, V


# --------------------------------------------------------------------------
# The reference itself (oracle/_ref), where it could be built.
# --------------------------------------------------------------------------
_R = None


def ref_available() -> bool:
    return os.path.exists(REF_LIB_PATH)


def ref_lib() -> C.CDLL:
    global _R
    if _R is None:
        R = C.CDLL(REF_LIB_PATH)
        R.fill_doci_data.argtypes = [C.c_char_p, C.POINTER(C.c_void_p)]
        R.doci_get_diagonal.argtypes = [C.c_void_p]
        R.doci_get_diagonal.restype = _pd
        R.doci_get_basis_size.argtypes = [C.c_void_p]
        R.doci_cleanup_data.argtypes = [C.POINTER(C.c_void_p)]
        R.doci_matvec.argtypes = [_pd, _pd, C.c_void_p]
        R.ref_to_bitstring.argtypes = [C.c_void_p]
        R.ref_to_bitstring.restype = C.POINTER(C.c_uint)
        R.ref_viikk.argtypes = [C.c_void_p]
        R.ref_viikk.restype = _pd
        R.ref_threadnos.argtypes = [C.c_void_p]
        R.davidson.argtypes = [_pd, _pd, C.c_int, C.c_int, C.c_double, C.c_void_p, _pd, C.c_int, C.c_int, C.c_void_p]
        R.ray_q.argtypes = [C.c_void_p, _pd, _pd, C.c_int, _pd, C.c_double, C.c_int, _pd, C.c_void_p]
        _R = R
    return _R


class RefHam:
    """The reference's own doci_data (fill_doci_data) through oracle/_ref."""

    def __init__(self, fcidump: str):
        self._d = C.c_void_p()
        ref_lib().fill_doci_data(os.fsencode(fcidump), C.byref(self._d))
        self.D = ref_lib().doci_get_basis_size(self._d)

    def close(self):
        if self._d:
            ref_lib().doci_cleanup_data(C.byref(self._d))

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def diag(self):
        return np.ctypeslib.as_array(ref_lib().doci_get_diagonal(self._d), (self.D,)).copy()

    @property
    def bitstrings(self):
        return np.ctypeslib.as_array(ref_lib().ref_to_bitstring(self._d), (self.D,)).astype(np.uint32)

    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        ref_lib().doci_matvec(_p(x), _p(y), self._d)
        return y
