"""Pins of the CPU oracle (oracle/) against the reference's own goldens.

* published energies / iteration counts of tests/coHF.out and tests/lifHF.out;
* the reference run on the golden cases (golden.json, sigma_*.npz, made by
  tests/golden/make_golden.py from oracle/_ref, the reference compiled from its
  sources);
* the reference itself, live, when oracle/_ref is built in this checkout;
* an independent dense Hamiltonian for small L.
"""
import itertools
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

SMALL = ["H2O_STO3G", "N2_STO3G", "H2O_631G", "lili_321g", "synthetic_L14_N7_s1", "synthetic_L10_N5_s3"]


@pytest.mark.parametrize("name", SMALL)
def test_addressing_diag_sigma_vs_reference_fixture(name, fcidump):
    z = np.load(os.path.join(GOLDEN, f"sigma_{name}.npz"))
    h = oracle.Ham(fcidump(name))
    assert np.array_equal(oracle.bitstrings(h.L, h.N), z["bitstrings"])  # bit-exact lexical order
    for r in range(h.D):
        b = int(z["bitstrings"][r])
        assert oracle.lib().orc_rank(b, h.L, h.N) == r
        assert oracle.lib().orc_unrank(r, h.L, h.N) == b
    assert np.array_equal(h.diag, z["diag"])  # same summation order -> bit-identical
    y = h.matvec(z["x"], nthreads=1)
    assert np.abs(y - z["sigma"]).max() <= 1e-12 * np.abs(z["sigma"]).max()


@pytest.mark.parametrize("name", SMALL + ["lif_631g_1"])
def test_davidson_energy_and_iterations_vs_reference(name, fcidump, golden):
    g = golden["cases"][name]
    h = oracle.Ham(fcidump(name))
    res, _ = h.davidson(tol=1e-8, max_its=1000)
    assert abs(res["energy"] - g["davidson"]["energy"]) < 1e-8
    assert res["iterations"] == len(g["D_exe"]["trace"])
    # the per-iteration residual trace follows the reference's
    ref = np.array([t[1] for t in g["D_exe"]["trace"]])
    assert np.allclose(res["trace"][:, 0], ref, rtol=1e-3, atol=1e-12)


def test_published_lif_energy(fcidump, golden):
    pub = golden["published"]["lif_631g_1"]
    h = oracle.Ham(fcidump("lif_631g_1"))
    res, _ = h.davidson(tol=1e-8, max_its=1000)
    assert round(res["energy"], 10) == pytest.approx(pub["energy"], abs=1e-10)
    assert res["iterations"] == pub["iterations"]


@pytest.mark.parametrize("name", ["synthetic_L10_N5_s3", "H2O_631G", "N2_STO3G"])
@pytest.mark.parametrize("precond", [False, True])
def test_ray_q_vs_reference(name, precond, fcidump, golden):
    g = golden["cases"][name]["CGP_exe" if precond else "CG_exe"]
    h = oracle.Ham(fcidump(name))
    res, _ = h.ray_q(tol=1e-8, max_its=60, precond=precond)
    # the reference prints the energy with %f per iteration and %.10lf at the end
    assert abs(res["energy"] - g["energy_printed"]) < 2e-9
    its_ref = len(g["trace"]) - 1  # first printed row is the start
    assert res["iterations"] == its_ref


def test_dense_hamiltonian_independent():
    """sigma = H x with H built from the DOCI formula (no reference code)."""
    from doci_gb300.fcidump import write_synthetic_fcidump, synthetic_integrals
    import tempfile
    L, N, seed = 8, 4, 11
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "s.FCIDUMP")
        write_synthetic_fcidump(p, L, N, seed)
        o = oracle.Ham(p)
        hmat, eri = synthetic_integrals(L, seed)
        dets = [c for c in itertools.combinations(range(L), N)]
        D = len(dets)
        H = np.zeros((D, D))
        index = {c: r for r, c in enumerate(dets)}
        for r, c in enumerate(dets):
            s = set(c)
            e = sum(2 * hmat[i, i] + eri[i, i, i, i] for i in c)
            e += sum(2 * eri[i, i, j, j] - eri[i, j, j, i] for i in c for j in c if j != i)
            H[r, r] = e
            for i in c:
                for a in range(L):
                    if a in s:
                        continue
                    t = tuple(sorted((s - {i}) | {a}))
                    H[r, index[t]] = eri[i, a, i, a]
        assert np.allclose(H, H.T)
        x = np.random.default_rng(0).standard_normal(D)
        assert np.abs(o.matvec(x) - H @ x).max() < 1e-12 * np.abs(H @ x).max()
        assert np.abs(o.diag - np.diag(H)).max() < 1e-12


def test_jacobi_matches_eigh():
    rng = np.random.default_rng(3)
    for n in (1, 2, 5, 17, 30):
        A = rng.standard_normal((n, n))
        A = A + A.T
        w, V = oracle.jacobi_eig(A)
        assert np.allclose(w, np.linalg.eigvalsh(A), atol=1e-12)
        assert np.allclose(A @ V, V * w, atol=1e-10)


@pytest.mark.skipif(not oracle.ref_available(), reason="oracle/_ref not built (no reference checkout)")
@pytest.mark.parametrize("L,N,seed", [(12, 6, 5), (16, 3, 6), (9, 8, 2)])
def test_oracle_vs_live_reference(L, N, seed, synth):
    p = synth(L, N, seed)
    o, r = oracle.Ham(p), oracle.RefHam(p)
    assert np.array_equal(oracle.bitstrings(L, N), r.bitstrings)
    assert np.array_equal(o.diag, r.diag)
    x = np.random.default_rng(seed).standard_normal(o.D)
    y0, y1 = r.matvec(x), o.matvec(x)
    assert np.abs(y0 - y1).max() <= 1e-12 * np.abs(y0).max()


def test_gather_rows_matches_matvec(synth):
    p = synth(13, 6, 4)
    o = oracle.Ham(p)
    x = np.random.default_rng(1).standard_normal(o.D)
    y = o.matvec(x)
    first = np.array([0, 100, o.D - 50], dtype=np.uint64)
    length = np.array([30, 200, 50], dtype=np.uint64)
    rows = np.concatenate([np.arange(f, f + n) for f, n in zip(first, length)]).astype(np.int64)
    yr = o.gather_rows(x, first, length, o.diag[rows])
    assert np.abs(yr - y[rows]).max() <= 1e-12 * np.abs(y).max()


@pytest.mark.parametrize("L,N,seed", [(20, 10, 41), (22, 6, 42)])
def test_gather_rows_matches_matvec_whole_space(L, N, seed, synth):
    """The gather form (prefix-sum neighbour ranks) that checks the sampled
    rows of the full-size GPU tests, against the reference-order matvec
    (direct ranks, symmetric scatter, doci.c:164-238) on every row of a
    mid-size space."""
    p = synth(L, N, seed)
    o = oracle.Ham(p)
    x = np.random.default_rng(seed).standard_normal(o.D)
    y = o.matvec(x)
    first = np.array([0], dtype=np.uint64)
    length = np.array([o.D], dtype=np.uint64)
    yr = o.gather_rows(x, first, length, o.diag)
    assert np.abs(yr - y).max() <= 1e-12 * np.abs(y).max()
