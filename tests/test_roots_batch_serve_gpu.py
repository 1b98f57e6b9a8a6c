"""Several roots (block Davidson), batched solves and the request server.

Roots 2-4 have no reference counterpart (the reference is single-root): they
are checked against a dense diagonalisation of the Hamiltonian built column
by column from the oracle's matvec; the lowest root against the reference's
golden energy.  Batched results must be bit-identical to the same solve run
alone; served one-root results equal the same single-root solve run alone to
1e-9 Ha."""
import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dg():
    import doci_gb300
    doci_gb300.lib()
    return doci_gb300


def dense_eigs(path, k):
    o = oracle.Ham(path)
    H = np.empty((o.D, o.D))
    e = np.zeros(o.D)
    for c in range(o.D):
        e[c] = 1.0
        H[:, c] = o.matvec(e, nthreads=1)
        e[c] = 0.0
    return np.linalg.eigvalsh(0.5 * (H + H.T))[:k]


@pytest.mark.parametrize("mode", ["fp64", "mixed"])
@pytest.mark.parametrize("L,N,seed", [(12, 6, 51), (13, 5, 52), (14, 7, 1)])
def test_four_roots_vs_dense(L, N, seed, mode, synth, dg):
    p = synth(L, N, seed)
    ref = dense_eigs(p, 4)
    with dg.Hamiltonian.from_fcidump(p) as h:
        r = dg.solve_roots(h, nroots=4, tol=1e-7, mode=mode, max_vec=20)
    assert r["status"] == 0 and r["converged"] == 1
    assert np.allclose(r["energies"], ref, atol=1e-9), (r["energies"], ref)
    assert max(r["residuals"]) <= 1e-7


def test_lowest_root_matches_reference(fcidump, golden, dg):
    name = "synthetic_L14_N7_s1"
    with dg.Hamiltonian.from_fcidump(fcidump(name)) as h:
        r = dg.solve_roots(h, nroots=2, tol=1e-7, mode="mixed")
    assert abs(r["energies"][0] - golden["cases"][name]["davidson"]["energy"]) < 1e-8


def test_batch_same_as_alone(synth, dg):
    specs = [(L, L // 2 + d, 100 + i) for i, (L, d) in enumerate([(10, 0), (12, -1), (16, 0), (11, 1), (14, 0),
                                                                    (18, 0), (13, 0), (15, -2), (12, 0), (17, 1)])]
    hams = [dg.Hamiltonian.from_fcidump(synth(*s)) for s in specs]
    try:
        alone = [dg.solve_roots(h, nroots=4, tol=1e-6, mode="mixed") for h in hams]
        st, mixed = dg.batch_solve(hams, nroots=4, tol=1e-6, mode="mixed", workers=6)
        assert st == 0
        for a, b in zip(alone, mixed):
            assert a["energies"] == b["energies"]  # bit-identical
            assert a["iterations"] == b["iterations"]
    finally:
        for h in hams:
            h.close()


def test_server_continuous_batching(dg):
    from doci_gb300.fcidump import raw_integrals
    rng = np.random.default_rng(4)
    reqs = []
    for i in range(14):
        L = int(rng.integers(10, 19))
        N = L // 2 + int(rng.integers(-2, 3))
        reqs.append((L, N, 2000 + i))
    alone = {}
    for L, N, seed in reqs:
        one, two = raw_integrals(L, seed)
        with dg.Hamiltonian.from_integrals(L, N, 0.0, one, two) as h:
            # a one-root request runs the single-root device Davidson with the
            # server's options (doci_batch_opts defaults: MAX_VEC 16, mixed_tol 1e-4)
            r, _ = h.solve(solver="D", tol=1e-6, mode="mixed", mixed_tol=1e-4, davidson_max_vec=16,
                           davidson_keep=2, max_its=200)
            alone[seed] = r
    with dg.Server(nroots=1, tol=1e-6, mode="mixed", workers=5) as srv:
        tickets = {}
        for L, N, seed in reqs:
            one, two = raw_integrals(L, seed)
            tickets[seed] = srv.submit(L, N, one, two)
        st, _ = srv.poll(10_000)
        assert st == 10  # DOCI_ERR_NOT_FOUND
        results = {seed: srv.wait(t) for seed, t in tickets.items()}
        s = srv.stats()
        assert s["submitted"] == s["finished"] == len(reqs) and s["bytes_in_use"] == 0
    overlapped = 0
    for seed, r in results.items():
        assert r["status"] == 0 and r["converged"] == 1
        # same alone and in the mix, within the rounding of the FP32 sigma's atomic adds
        assert abs(r["energies"][0] - alone[seed]["energy"]) <= 1e-9
        assert r["queued_s"] <= r["start_s"] <= r["end_s"]
        overlapped += any(o is not r and o["start_s"] < r["end_s"] and r["start_s"] < o["end_s"]
                          for o in results.values())
    assert overlapped > 0  # requests ran concurrently


def test_server_admission_rejects_oversized(dg):
    from doci_gb300.fcidump import raw_integrals
    one, two = raw_integrals(12, 7)
    with dg.Server(nroots=1, workers=1, hbm_budget=1 << 20) as srv:
        t = srv.submit(12, 6, one, two)
        r = srv.wait(t)
    assert r["status"] == 9  # DOCI_ERR_ADMISSION


def test_engine_tile_autotune(synth, dg):
    """doci_engine_autotune picks, for one (L, N) shape, the batch engine's
    sigma path: a tile of 1, 2 or 4 determinants per thread of the batched
    gather (returned as 1, 2, 4), or the single-problem kernels (returned as
    0).  A tile shape changes which thread computes a determinant, not its
    sum; the single-problem kernels reduce in another order.  Either way the
    solve reaches the same energies, within the residual tolerance's
    quadratic energy error."""
    with dg.Hamiltonian.from_fcidump(synth(16, 8, 61)) as h:
        before = dg.solve_roots(h, nroots=2, tol=1e-6, mode="mixed")
        choice = h.engine_autotune(2)
        assert choice in (0, 1, 2, 4)
        after = dg.solve_roots(h, nroots=2, tol=1e-6, mode="mixed")
    assert before["converged"] == after["converged"] == 1
    assert np.allclose(before["energies"], after["energies"], rtol=0, atol=1e-9)
