"""ctypes binding of libdoci_gb300.so (the C ABI declared in include/doci_gb300.h).

The shared library is the product; this module only loads it and converts
numpy arrays / torch device tensors to the plain pointers the C ABI takes.
Nothing here computes: if the library is missing the import fails loudly.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libdoci_gb300.so")

FP64, FP32 = 0, 1
SOLVER_D, SOLVER_CG, SOLVER_CGP = 0, 1, 2
MODE_FP64, MODE_MIXED = 0, 1
_SOLVERS = {"D": SOLVER_D, "CG": SOLVER_CG, "CGP": SOLVER_CGP}

STATUS = {
    0: "DOCI_OK", 1: "DOCI_ERR_OPEN", 2: "DOCI_ERR_FORMAT", 3: "DOCI_ERR_NALPHA_NBETA",
    4: "DOCI_ERR_TOO_MANY_ORBITALS", 5: "DOCI_ERR_INVALID", 6: "DOCI_ERR_CUDA",
    7: "DOCI_ERR_OUT_OF_MEMORY", 8: "DOCI_ERR_NO_DEVICE", 9: "DOCI_ERR_ADMISSION",
    10: "DOCI_ERR_NOT_FOUND", 11: "DOCI_ERR_PENDING", 12: "DOCI_ERR_DEVICE_TIMEOUT",
    13: "DOCI_ERR_UNKNOWN_SOLVER",
}


class DociError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        self.name = STATUS.get(status, str(status))
        msg = lib().doci_status_string(status).decode() if _LIB is not None else self.name
        super().__init__(f"{what}: {self.name} ({msg})" if what else f"{self.name} ({msg})")


class SolveOpts(C.Structure):
    _fields_ = [
        ("solver", C.c_int), ("max_its", C.c_int), ("tol", C.c_double),
        ("davidson_keep", C.c_int), ("davidson_max_vec", C.c_int), ("hf_init", C.c_int),
        ("mode", C.c_int), ("mixed_tol", C.c_double), ("print_level", C.c_int),
        ("seed", C.c_uint64), ("fp32_corrections", C.c_int),
    ]


class SolveResult(C.Structure):
    _fields_ = [
        ("energy", C.c_double), ("residual", C.c_double), ("iterations", C.c_int),
        ("iterations_fp32", C.c_int), ("converged", C.c_int), ("status_code", C.c_int),
        ("energy_fp32", C.c_double), ("seconds", C.c_double), ("sigma_seconds", C.c_double),
    ]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchOpts(C.Structure):
    _fields_ = [("nroots", C.c_int), ("max_vec", C.c_int), ("max_its", C.c_int), ("tol", C.c_double),
                ("mode", C.c_int), ("mixed_tol", C.c_double), ("workers", C.c_int), ("hbm_budget", C.c_int64),
                ("keep", C.c_int)]


class RootResult(C.Structure):
    _fields_ = [("energy", C.c_double * 8), ("residual", C.c_double * 8), ("energy_fp32", C.c_double * 8),
                ("nroots", C.c_int), ("iterations", C.c_int), ("iterations_fp32", C.c_int), ("sigmas", C.c_int),
                ("converged", C.c_int), ("status", C.c_int), ("queued_s", C.c_double), ("start_s", C.c_double),
                ("end_s", C.c_double)]

    def as_dict(self):
        n = self.nroots
        return {"energies": list(self.energy[:n]), "residuals": list(self.residual[:n]),
                "energies_fp32": list(self.energy_fp32[:n]), "iterations": self.iterations,
                "iterations_fp32": self.iterations_fp32, "sigmas": self.sigmas, "converged": self.converged,
                "status": self.status, "queued_s": self.queued_s, "start_s": self.start_s, "end_s": self.end_s}


_LIB = None
MATVEC_FN = C.CFUNCTYPE(None, C.POINTER(C.c_double), C.POINTER(C.c_double), C.c_void_p)


def lib() -> C.CDLL:
    """Load libdoci_gb300.so once; raise if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise ImportError(
            f"{LIB_PATH} is missing: build it with `python -m doci_gb300.build` "
            "(there is no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    vp, i, d, i64 = C.c_void_p, C.c_int, C.c_double, C.c_int64
    pd = C.POINTER(C.c_double)
    sig = {
        "doci_status_string": (C.c_char_p, [i]),
        "doci_ham_from_fcidump": (i, [C.c_char_p, C.POINTER(vp)]),
        "doci_ham_from_fcidump_relaxed": (i, [C.c_char_p, C.POINTER(vp)]),
        "doci_fcidump_integrals": (i, [C.c_char_p, i, C.POINTER(i), C.POINTER(i), C.POINTER(i), pd, pd, pd,
                                       C.POINTER(i)]),
        "doci_ham_from_integrals": (i, [i, i, d, pd, pd, C.POINTER(vp)]),
        "doci_ham_destroy": (None, [vp]),
        "doci_ham_dims": (i, [vp, C.POINTER(i), C.POINTER(i), C.POINTER(i64)]),
        "doci_ham_diagonal": (i, [vp, pd]),
        "doci_ham_diagonal_device": (vp, [vp]),
        "doci_sigma": (i, [vp, vp, vp, i, vp]),
        "doci_sigma_block": (i, [vp, vp, C.c_int64, vp, C.c_int64, i, i, vp]),
        "doci_sigma_plan": (i, [vp, i, C.POINTER(i), C.POINTER(i)]),
        "doci_ham_autotune": (i, [vp, i, i, C.POINTER(i)]),
        "doci_sigma_host": (i, [vp, vp, vp, i]),
        "doci_engine_autotune": (i, [vp, i, vp]),
        "doci_ham_set_sigma_kernel": (i, [vp, i]),
        "doci_bitstrings": (i, [vp, i64, i64, vp, vp]),
        "doci_ranks": (i, [vp, vp, i64, vp, vp]),
        "doci_multidot": (i, [vp, i64, i, vp, i64, i, vp, vp]),
        "doci_solve_opts_default": (None, [C.POINTER(SolveOpts)]),
        "doci_solve": (i, [vp, C.POINTER(SolveOpts), pd, C.POINTER(SolveResult)]),
        "doci_solve_footprint": (i64, [i, i, C.POINTER(SolveOpts), i]),
        "doci_solve_trace": (i, [vp, C.POINTER(SolveOpts), pd, C.POINTER(SolveResult), pd, i, C.POINTER(i)]),
        "doci_batch_opts_default": (None, [C.POINTER(BatchOpts)]),
        "doci_roots_footprint": (i64, [i, i, C.POINTER(BatchOpts)]),
        "doci_solve_roots": (i, [vp, C.POINTER(BatchOpts), C.POINTER(RootResult), pd]),
        "doci_batch_solve": (i, [i, C.POINTER(vp), C.POINTER(BatchOpts), C.POINTER(RootResult)]),
        "doci_server_create": (i, [C.POINTER(BatchOpts), C.POINTER(vp)]),
        "doci_server_submit": (i, [vp, i, i, d, pd, pd, C.POINTER(i64)]),
        "doci_server_submit_fcidump": (i, [vp, C.c_char_p, C.POINTER(i64)]),
        "doci_server_poll": (i, [vp, i64, C.POINTER(RootResult)]),
        "doci_server_wait": (i, [vp, i64, C.POINTER(RootResult)]),
        "doci_server_stats": (i, [vp, C.POINTER(i64), C.POINTER(i64), C.POINTER(i64), C.POINTER(i64)]),
        "doci_server_destroy": (None, [vp]),
        # reference-compatible drop-in
        "fill_doci_data": (None, [C.c_char_p, C.POINTER(vp)]),
        "doci_get_diagonal": (pd, [vp]),
        "doci_get_basis_size": (i, [vp]),
        "doci_cleanup_data": (None, [C.POINTER(vp)]),
        "doci_matvec": (None, [pd, pd, vp]),
        "sparse_eigensolve": (i, [pd, i, pd, vp, pd, pd, d, i, C.c_char_p, i, i, vp]),
        "davidson": (i, [pd, pd, i, i, d, vp, pd, i, i, vp]),
        "ray_q": (i, [vp, pd, pd, i, pd, d, i, pd, vp]),
        "read_fcidump": (None, [C.c_char_p, C.POINTER(C.c_uint), C.POINTER(C.c_uint),
                                C.POINTER(C.c_uint), pd, C.POINTER(pd), C.POINTER(pd)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _LIB = L
    return L


def _check(st: int, what: str) -> None:
    if st != 0:
        raise DociError(st, what)


def _dptr(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def default_opts(**kw) -> SolveOpts:
    o = SolveOpts()
    lib().doci_solve_opts_default(C.byref(o))
    for k, v in kw.items():
        if k == "solver" and isinstance(v, str):
            v = _SOLVERS[v]
        if k == "mode" and isinstance(v, str):
            v = {"fp64": MODE_FP64, "mixed": MODE_MIXED}[v]
        setattr(o, k, v)
    return o


KERNEL_KINDS = {"auto": 0, "gather": 1, "row1": 3, "rowx": 4, "pair": 6, "tc": 8, "rowff": 9}
KERNEL_NAMES = {v: k for k, v in KERNEL_KINDS.items()}


class Hamiltonian:
    """A DOCI Hamiltonian resident on the current CUDA device (doci_ham)."""

    def __init__(self, handle: int):
        self._h = C.c_void_p(handle)
        L, N, D = C.c_int(), C.c_int(), C.c_int64()
        _check(lib().doci_ham_dims(self._h, C.byref(L), C.byref(N), C.byref(D)), "doci_ham_dims")
        self.L, self.N, self.D = L.value, N.value, D.value

    @classmethod
    def from_fcidump(cls, path: str, relaxed: bool = False) -> "Hamiltonian":
        """relaxed=True: the relaxed reader (any namelist layout and integral
        index order); default: the reference's reader."""
        h = C.c_void_p()
        fn = lib().doci_ham_from_fcidump_relaxed if relaxed else lib().doci_ham_from_fcidump
        _check(fn(os.fsencode(path), C.byref(h)), f"doci_ham_from_fcidump({path})")
        return cls(h.value)

    @classmethod
    def from_integrals(cls, L: int, n_pairs: int, core: float, one: np.ndarray, two: np.ndarray):
        one = np.ascontiguousarray(one, dtype=np.float64).reshape(-1)
        two = np.ascontiguousarray(two, dtype=np.float64).reshape(-1)
        h = C.c_void_p()
        _check(lib().doci_ham_from_integrals(L, n_pairs, core, _dptr(one), _dptr(two), C.byref(h)),
               "doci_ham_from_integrals")
        return cls(h.value)

    @property
    def handle(self) -> C.c_void_p:
        return self._h

    def close(self) -> None:
        if self._h is not None and self._h.value:
            lib().doci_ham_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def engine_autotune(self, nvec: int = 1) -> int:
        """The batch engine's sigma path for this shape, timed and kept for
        the process: 1, 2 or 4 determinants per thread of the batched gather,
        or 0 for the single-problem kernels; doci_engine_autotune."""
        d = C.c_int()
        _check(lib().doci_engine_autotune(self._h, int(nvec), C.byref(d)), "doci_engine_autotune")
        return d.value

    def set_sigma_kernel(self, kind) -> None:
        """0/'auto', 1/'gather', 3/'row1' (row pass), 4/'rowx' (phase-ordered row pass),
        6/'pair' (pair form, mma.sync), 8/'tc' (pair form, tcgen05), 9/'rowff' (FP64 float-float row
        pass); doci_ham_set_sigma_kernel."""
        kind = KERNEL_KINDS.get(kind, kind)
        _check(lib().doci_ham_set_sigma_kernel(self._h, int(kind)), "doci_ham_set_sigma_kernel")

    def diagonal(self) -> np.ndarray:
        out = np.empty(self.D, dtype=np.float64)
        _check(lib().doci_ham_diagonal(self._h, _dptr(out)), "doci_ham_diagonal")
        return out

    def diagonal_device_ptr(self) -> int:
        return lib().doci_ham_diagonal_device(self._h)

    def sigma(self, x: np.ndarray, precision: int = FP64) -> np.ndarray:
        """sigma = H x for a host vector (copies in and out inside the call)."""
        dt = np.float64 if precision == FP64 else np.float32
        x = np.ascontiguousarray(x, dtype=dt)
        if x.shape != (self.D,):
            raise ValueError(f"x must have shape ({self.D},)")
        y = np.empty_like(x)
        _check(lib().doci_sigma_host(self._h, x.ctypes.data, y.ctypes.data, precision), "doci_sigma_host")
        return y

    def sigma_device(self, x_ptr: int, y_ptr: int, precision: int = FP64, stream: int = 0) -> None:
        """sigma on device buffers (e.g. torch tensors' data_ptr())."""
        _check(lib().doci_sigma(self._h, C.c_void_p(x_ptr), C.c_void_p(y_ptr), precision,
                                C.c_void_p(stream or None)), "doci_sigma")

    def autotune(self, precision: int = FP32, nvec: int = 1) -> int:
        """Time the sigma paths for this shape and keep the fastest (process-wide)."""
        c = C.c_int()
        _check(lib().doci_ham_autotune(self._h, precision, nvec, C.byref(c)), "doci_ham_autotune")
        return c.value

    def sigma_plan(self, precision: int = FP64):
        """(kind, launches) of doci_sigma on this handle: the kernel the
        automatic choice resolves to and the kernel launches per call."""
        k, n = C.c_int(), C.c_int()
        _check(lib().doci_sigma_plan(self._h, precision, C.byref(k), C.byref(n)), "doci_sigma_plan")
        return k.value, n.value

    def sigma_block_device(self, x_ptr: int, ldx: int, y_ptr: int, ldy: int, nv: int, precision: int = FP64,
                           stream: int = 0) -> None:
        """Block sigma over nv column-major vectors on device buffers."""
        _check(lib().doci_sigma_block(self._h, C.c_void_p(x_ptr), ldx, C.c_void_p(y_ptr), ldy, nv, precision,
                                      C.c_void_p(stream or None)), "doci_sigma_block")

    def bitstrings_device(self, first: int, count: int, out_ptr: int, stream: int = 0) -> None:
        _check(lib().doci_bitstrings(self._h, first, count, C.c_void_p(out_ptr), C.c_void_p(stream or None)),
               "doci_bitstrings")

    def ranks_device(self, bits_ptr: int, count: int, out_ptr: int, stream: int = 0) -> None:
        _check(lib().doci_ranks(self._h, C.c_void_p(bits_ptr), count, C.c_void_p(out_ptr),
                                C.c_void_p(stream or None)), "doci_ranks")

    def solve(self, vec: np.ndarray | None = None, **opts):
        """Device-resident solve; returns (result dict, eigenvector)."""
        o = default_opts(**opts)
        v = np.empty(self.D, dtype=np.float64) if vec is None else np.ascontiguousarray(vec, dtype=np.float64).copy()
        if vec is not None and "hf_init" not in opts:
            o.hf_init = -1
        r = SolveResult()
        _check(lib().doci_solve(self._h, C.byref(o), _dptr(v), C.byref(r)), "doci_solve")
        return r.as_dict(), v


    def solve_trace(self, vec=None, max_records: int = 4096, **opts):
        """doci_solve with per-iteration records: returns (result, vector,
        trace array of rows (phase, residual, energy, seconds))."""
        o = default_opts(**opts)
        v = np.empty(self.D, dtype=np.float64) if vec is None else np.ascontiguousarray(vec, dtype=np.float64).copy()
        if vec is not None and "hf_init" not in opts:
            o.hf_init = -1
        r = SolveResult()
        tr = np.zeros((max_records, 4))
        n = C.c_int()
        _check(lib().doci_solve_trace(self._h, C.byref(o), _dptr(v), C.byref(r), _dptr(tr), max_records,
                                      C.byref(n)), "doci_solve_trace")
        return r.as_dict(), v, tr[:n.value].copy()


def fcidump_integrals(path: str, relaxed: bool = False) -> dict:
    """Raw integrals of an FCIDUMP (before the transform) by the reference's
    reader or the relaxed one; host only (no GPU needed)."""
    L, na, nb, bad = C.c_int(), C.c_int(), C.c_int(), C.c_int()
    core = C.c_double()
    p = os.fsencode(path)
    _check(lib().doci_fcidump_integrals(p, int(relaxed), C.byref(L), C.byref(na), C.byref(nb), C.byref(core),
                                        None, None, C.byref(bad)), f"doci_fcidump_integrals({path})")
    one = np.zeros(L.value ** 2)
    two = np.zeros(L.value ** 4)
    _check(lib().doci_fcidump_integrals(p, int(relaxed), None, None, None, None, _dptr(one), _dptr(two),
                                        C.byref(bad)), f"doci_fcidump_integrals({path})")
    return {"L": L.value, "n_alpha": na.value, "n_beta": nb.value, "core": core.value, "one": one, "two": two}


def batch_opts(**kw) -> BatchOpts:
    o = BatchOpts()
    lib().doci_batch_opts_default(C.byref(o))
    for k, v in kw.items():
        if k == "mode" and isinstance(v, str):
            v = {"fp64": MODE_FP64, "mixed": MODE_MIXED}[v]
        setattr(o, k, v)
    return o


def solve_roots(ham: "Hamiltonian", vectors: bool = False, **kw):
    o = batch_opts(**kw)
    r = RootResult()
    v = np.empty((o.nroots, ham.D)) if vectors else None
    _check(lib().doci_solve_roots(ham.handle, C.byref(o), C.byref(r), _dptr(v) if vectors else None),
           "doci_solve_roots")
    return (r.as_dict(), v) if vectors else r.as_dict()


def batch_solve(hams, **kw):
    o = batch_opts(**kw)
    arr = (C.c_void_p * len(hams))(*[h.handle.value for h in hams])
    res = (RootResult * len(hams))()
    st = lib().doci_batch_solve(len(hams), arr, C.byref(o), res)
    return st, [r.as_dict() for r in res]


class Server:
    """The request server (doci_server_*): submit integrals, get tickets."""

    def __init__(self, **kw):
        self._o = batch_opts(**kw)
        self._s = C.c_void_p()
        _check(lib().doci_server_create(C.byref(self._o), C.byref(self._s)), "doci_server_create")

    def submit(self, L, n_pairs, one, two, core=0.0) -> int:
        one = np.ascontiguousarray(one, dtype=np.float64).reshape(-1)
        two = np.ascontiguousarray(two, dtype=np.float64).reshape(-1)
        t = C.c_int64()
        _check(lib().doci_server_submit(self._s, L, n_pairs, core, _dptr(one), _dptr(two), C.byref(t)),
               "doci_server_submit")
        return t.value

    def submit_fcidump(self, path) -> int:
        t = C.c_int64()
        _check(lib().doci_server_submit_fcidump(self._s, os.fsencode(path), C.byref(t)), "doci_server_submit_fcidump")
        return t.value

    def poll(self, ticket):
        r = RootResult()
        st = lib().doci_server_poll(self._s, ticket, C.byref(r))
        return st, (r.as_dict() if st == 0 else None)

    def wait(self, ticket):
        r = RootResult()
        _check(lib().doci_server_wait(self._s, ticket, C.byref(r)), "doci_server_wait")
        return r.as_dict()

    def stats(self):
        v = [C.c_int64() for _ in range(4)]
        _check(lib().doci_server_stats(self._s, *[C.byref(x) for x in v]), "doci_server_stats")
        return dict(zip(("submitted", "finished", "running", "bytes_in_use"), [x.value for x in v]))

    def close(self):
        if self._s:
            lib().doci_server_destroy(self._s)
            self._s = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def footprint(L: int, n_pairs: int, nroots: int = 1, **opts) -> int:
    o = default_opts(**opts)
    return lib().doci_solve_footprint(L, n_pairs, C.byref(o), nroots)
