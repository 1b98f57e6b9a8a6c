"""The plain FP64 GPU solvers on the L=28, N=14 Hamiltonian (seed 2,
D = 40,116,600) against the reference executable's own runs of the same
FCIDUMP (tests/golden/golden.json "synthetic_L28_N14_s2", made by
tests/golden/make_golden.py --l28 from the reference compiled from its
sources): Davidson with DAVIDSON_MAX_VEC 30, DAVIDSON_KEEP 2, TOL 1e-8 and
the HF start (davidson.c:33-128), and CGP with MAX_ITS 40 (CG.c:13-164),
both dispatched as wrapper_solvers.c:15-20 does.

Davidson: the same energy (1e-8 Ha of the printed 10 decimals), the same
iteration count, and every iteration's printed energy (%f, one unit of the
last digit) and residue (%e; 1e-3 relative: GPU and CPU round differently in
the residual's cancellation).  CGP: the same energy (2e-9 of the printed
value), iteration count and return code."""
import pytest

pytestmark = pytest.mark.gpu

CASE = "synthetic_L28_N14_s2"


@pytest.fixture(scope="module")
def dg():
    import doci_gb300
    doci_gb300.lib()
    return doci_gb300


def test_l28_davidson_fp64(synth, golden, dg):
    g = golden["cases"][CASE]["D_exe"]
    with dg.Hamiltonian.from_fcidump(synth(28, 14, 2)) as h:
        assert h.D == golden["cases"][CASE]["D"]
        r, _, tr = h.solve_trace(solver="D", tol=1e-8, max_its=1000, davidson_max_vec=30, davidson_keep=2,
                                 mode="fp64")
    assert abs(r["energy"] - g["energy_printed"]) < 1e-8
    assert r["iterations"] == len(g["trace"])
    assert r["converged"] == 1 and r["status_code"] == g["exit_code"]
    for (it, res, e), row in zip(g["trace"], tr):
        assert abs(row[2] - e) <= 1.01e-6, (it, row[2], e)
        assert abs(row[1] - res) <= max(1e-3 * res, 1e-13), (it, row[1], res)


def test_l28_cgp(synth, golden, dg):
    g = golden["cases"][CASE]["CGP_exe"]
    with dg.Hamiltonian.from_fcidump(synth(28, 14, 2)) as h:
        r, _ = h.solve(solver="CGP", tol=1e-8, max_its=40)
    assert abs(r["energy"] - g["energy_printed"]) < 2e-9
    assert r["iterations"] == len(g["trace"]) - 1
    assert r["status_code"] == g["exit_code"]
