"""Device-resident Davidson and RQ-CG against the reference's goldens, and the
reference-compatible entry points (fill_doci_data / sparse_eigensolve)."""
import ctypes as C

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

CASES = ["H2O_STO3G", "N2_STO3G", "H2O_631G", "lili_321g", "synthetic_L14_N7_s1", "synthetic_L10_N5_s3",
         "lif_631g_1"]


@pytest.fixture(scope="module")
def dg():
    import doci_gb300
    doci_gb300.lib()
    return doci_gb300


@pytest.mark.parametrize("name", CASES)
def test_davidson_vs_reference(name, fcidump, golden, dg):
    g = golden["cases"][name]
    with dg.Hamiltonian.from_fcidump(fcidump(name)) as h:
        r, x = h.solve(solver="D", tol=1e-8, max_its=1000)
    assert abs(r["energy"] - g["davidson"]["energy"]) < 1e-8
    assert r["iterations"] == len(g["D_exe"]["trace"])
    assert r["converged"] == 1 and r["status_code"] == 0
    assert abs(np.linalg.norm(x) - 1) < 1e-10


def test_published_co_and_lif(fcidump, golden, dg):
    for name in ("co_631g_1", "lif_631g_1"):
        pub = golden["published"][name]
        with dg.Hamiltonian.from_fcidump(fcidump(name)) as h:
            r, _ = h.solve(solver="D", tol=1e-8, max_its=1000)
        assert round(r["energy"], 10) == pytest.approx(pub["energy"], abs=1e-10), name
        assert r["iterations"] == pub["iterations"], name


@pytest.mark.parametrize("name", ["synthetic_L10_N5_s3", "H2O_631G", "N2_STO3G"])
@pytest.mark.parametrize("solver", ["CG", "CGP"])
def test_ray_q_vs_reference(name, solver, fcidump, golden, dg):
    g = golden["cases"][name][solver + "_exe"]
    with dg.Hamiltonian.from_fcidump(fcidump(name)) as h:
        r, _ = h.solve(solver=solver, tol=1e-8, max_its=60)
    assert abs(r["energy"] - g["energy_printed"]) < 2e-9
    assert r["iterations"] == len(g["trace"]) - 1
    assert r["status_code"] == 1  # CG.c:163 returns its <= max_its


def test_deflation_and_small_subspace(synth, dg):
    p = synth(16, 8, 41)
    o = oracle.Ham(p)
    ref, _ = o.davidson(max_vectors=6, keep=3, tol=1e-9, max_its=500)
    with dg.Hamiltonian.from_fcidump(p) as h:
        r, _ = h.solve(solver="D", tol=1e-9, max_its=500, davidson_max_vec=6, davidson_keep=3)
    assert abs(r["energy"] - ref["energy"]) < 1e-9
    assert r["iterations"] == ref["iterations"]


def test_mixed_precision_reaches_fp64_energy(synth, dg):
    p = synth(20, 10, 42)
    with dg.Hamiltonian.from_fcidump(p) as h:
        r64, _ = h.solve(solver="D", tol=1e-10, max_its=500)
        rm, _ = h.solve(solver="D", tol=1e-6, max_its=500, mode="mixed", mixed_tol=1e-4)
    assert rm["iterations_fp32"] > 0
    assert abs(rm["energy"] - r64["energy"]) < 1e-8


def test_dropin_entry_points(fcidump, golden, dg, capfd):
    """fill_doci_data + sparse_eigensolve(doci_matvec) exactly as executable.c calls them."""
    L = dg.lib()
    name = "H2O_631G"
    dat = C.c_void_p()
    L.fill_doci_data(fcidump(name).encode(), C.byref(dat))
    D = L.doci_get_basis_size(dat)
    diag = L.doci_get_diagonal(dat)
    d = np.ctypeslib.as_array(diag, (D,))
    vec = np.zeros(D)
    vec[int(np.argmin(d))] = 1.0
    e = C.c_double()
    mv = C.cast(L.doci_matvec, C.c_void_p)
    info = L.sparse_eigensolve(vec.ctypes.data_as(C.POINTER(C.c_double)), D, C.byref(e), mv, diag, None, 1e-8,
                               1000, b"D", 2, 30, dat)
    assert info == 0
    assert abs(e.value - golden["cases"][name]["davidson"]["energy"]) < 1e-8
    # doci_matvec on host buffers
    x = np.random.default_rng(0).standard_normal(D)
    y = np.empty(D)
    L.doci_matvec(x.ctypes.data_as(C.POINTER(C.c_double)), y.ctypes.data_as(C.POINTER(C.c_double)), dat)
    yr = oracle.Ham(fcidump(name)).matvec(x)
    assert np.abs(y - yr).max() <= 1e-12 * np.abs(yr).max()
    assert L.sparse_eigensolve(vec.ctypes.data_as(C.POINTER(C.c_double)), D, C.byref(e), mv, diag, None, 1e-8, 5,
                               b"XX", 2, 30, dat) == -1
    L.doci_cleanup_data(C.byref(dat))
    assert not dat.value
    out = capfd.readouterr().out
    assert "basis size : %d" % D in out and "DAVIDSON ITERATIONS" in out


def test_foreign_matvec_through_sparse_eigensolve(fcidump, golden, dg):
    """A matvec that is not doci_matvec is called on host buffers each iteration."""
    L = dg.lib()
    name = "N2_STO3G"
    o = oracle.Ham(fcidump(name))
    calls = []

    @dg._lib.MATVEC_FN
    def mv(xp, yp, _):
        x = np.ctypeslib.as_array(xp, (o.D,))
        y = np.ctypeslib.as_array(yp, (o.D,))
        y[:] = o.matvec(x.copy())
        calls.append(1)

    diag = o.diag
    vec = np.zeros(o.D)
    vec[int(np.argmin(diag))] = 1.0
    e = C.c_double()
    info = L.sparse_eigensolve(vec.ctypes.data_as(C.POINTER(C.c_double)), o.D, C.byref(e), C.cast(mv, C.c_void_p),
                               diag.ctypes.data_as(C.POINTER(C.c_double)), None, 1e-8, 1000, b"D", 2, 30, None)
    assert info == 0
    assert abs(e.value - golden["cases"][name]["davidson"]["energy"]) < 1e-8
    assert len(calls) == len(golden["cases"][name]["D_exe"]["trace"])


def test_solve_trace_records_both_phases(synth, dg):
    p = synth(18, 9, 43)
    with dg.Hamiltonian.from_fcidump(p) as h:
        r, _, tr = h.solve_trace(solver="D", tol=1e-8, max_its=300, mode="mixed", mixed_tol=1e-4)
        r64, _, tr64 = h.solve_trace(solver="D", tol=1e-8, max_its=300)
    assert len(tr) == r["iterations"] and len(tr64) == r64["iterations"]
    assert (tr[: r["iterations_fp32"], 0] == 0).all() and (tr[r["iterations_fp32"]:, 0] == 1).all()
    assert (tr64[:, 0] == 1).all()
    assert np.all(np.diff(tr[:, 3]) >= 0) and np.all(np.diff(tr64[:, 3]) >= 0)
    assert abs(tr[-1, 2] - r["energy"]) < 1e-12 and abs(tr64[-1, 2] - r64["energy"]) < 1e-12
    assert abs(r["energy"] - r64["energy"]) < 1e-8
