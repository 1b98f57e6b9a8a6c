"""GPU sigma / diagonal / addressing parity against the oracle and the
reference's golden fixtures.  Every call goes through the C ABI of
libdoci_gb300.so (doci_gb300._lib is a ctypes binding)."""
import os

import numpy as np
import pytest

import oracle
from conftest import GOLDEN

pytestmark = pytest.mark.gpu

SMALL = ["H2O_STO3G", "N2_STO3G", "H2O_631G", "lili_321g", "synthetic_L14_N7_s1", "synthetic_L10_N5_s3"]
# sigma tolerance: max|y_gpu - y_ref| <= tol * max|y_ref| (FP64 1e-12; FP32 storage/accumulation 2e-6)
TOL64, TOL32 = 1e-12, 2e-6


@pytest.fixture(scope="module")
def dg():
    import doci_gb300
    doci_gb300.lib()
    return doci_gb300


def torch_cuda():
    import torch
    assert torch.cuda.is_available()
    return torch


@pytest.mark.parametrize("name", SMALL)
def test_golden_sigma_diag_bits(name, fcidump, dg):
    z = np.load(os.path.join(GOLDEN, f"sigma_{name}.npz"))
    with dg.Hamiltonian.from_fcidump(fcidump(name)) as h:
        assert h.D == len(z["x"])
        assert np.array_equal(h.diagonal(), z["diag"])  # bit-identical to the reference
        y = h.sigma(z["x"], dg.FP64)
        assert np.abs(y - z["sigma"]).max() <= TOL64 * np.abs(z["sigma"]).max()
        y32 = h.sigma(z["x"].astype(np.float32), dg.FP32)
        assert np.abs(y32 - z["sigma"]).max() <= TOL32 * np.abs(z["sigma"]).max()
        torch = torch_cuda()
        bits = torch.empty(h.D, dtype=torch.int32, device="cuda")
        h.bitstrings_device(0, h.D, bits.data_ptr())
        torch.cuda.synchronize()
        assert np.array_equal(bits.cpu().numpy().view(np.uint32), z["bitstrings"])
        ranks = torch.empty(h.D, dtype=torch.int64, device="cuda")
        h.ranks_device(bits.data_ptr(), h.D, ranks.data_ptr())
        torch.cuda.synchronize()
        assert np.array_equal(ranks.cpu().numpy(), np.arange(h.D))


@pytest.mark.parametrize("kernel", ["auto", "gather", "row1", "rowx", "pair", "tc", "rowff"])
@pytest.mark.parametrize("L,N,seed", [(16, 8, 21), (18, 5, 22), (20, 10, 23), (12, 1, 24), (12, 11, 25),
                                      (7, 0, 26), (6, 6, 27), (32, 2, 28), (32, 30, 29), (24, 12, 30),
                                      (22, 11, 31), (26, 4, 32)])
def test_sigma_vs_oracle(L, N, seed, kernel, synth, dg):
    p = synth(L, N, seed)
    o = oracle.Ham(p)
    with dg.Hamiltonian.from_fcidump(p) as h:
        h.set_sigma_kernel(kernel)
        assert h.D == o.D
        assert np.array_equal(h.diagonal(), o.diag)
        x = np.random.default_rng(seed).standard_normal(h.D)
        yr = o.matvec(x)
        y = h.sigma(x, dg.FP64)
        assert np.abs(y - yr).max() <= TOL64 * np.abs(yr).max()
        y32 = h.sigma(x.astype(np.float32), dg.FP32)
        assert np.abs(y32 - yr).max() <= TOL32 * np.abs(yr).max()


def test_addressing_full_size_properties(synth, dg):
    """L=32, N=16 (D = 601,080,390): unrank -> rank round trip over sampled
    windows, lexical order (strictly increasing as 32-bit reversed strings is
    not the order; use the oracle's rank on samples instead)."""
    torch = torch_cuda()
    p = synth(32, 16, 3)
    with dg.Hamiltonian.from_fcidump(p) as h:
        assert h.D == 601080390
        for first in (0, 123456789, h.D - 4096, 300000000):
            n = min(4096, h.D - first)
            bits = torch.empty(n, dtype=torch.int32, device="cuda")
            h.bitstrings_device(first, n, bits.data_ptr())
            ranks = torch.empty(n, dtype=torch.int64, device="cuda")
            h.ranks_device(bits.data_ptr(), n, ranks.data_ptr())
            torch.cuda.synchronize()
            b = bits.cpu().numpy().view(np.uint32)
            assert np.array_equal(ranks.cpu().numpy(), np.arange(first, first + n))
            for k in range(0, n, 511):
                assert oracle.lib().orc_unrank(first + k, 32, 16) == b[k]
            assert all(bin(int(v)).count("1") == 16 for v in b[:64])


@pytest.mark.parametrize("kernel", ["auto", "gather", "row1", "rowx", "pair", "tc", "rowff"])
def test_sigma_full_size_symmetry_and_linearity(kernel, synth, dg):
    """L=28, N=14 (D = 40,116,600): H is symmetric, sigma is linear, and
    sampled rows agree with the oracle's gather form."""
    torch = torch_cuda()
    p = synth(28, 14, 2)
    o = oracle.Ham(p, keep_diag=False)
    with dg.Hamiltonian.from_fcidump(p) as h:
        h.set_sigma_kernel(kernel)
        D = h.D
        g = torch.Generator(device="cuda").manual_seed(7)
        x = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
        z = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
        hx = torch.empty_like(x)
        hz = torch.empty_like(x)
        h.sigma_device(x.data_ptr(), hx.data_ptr(), dg.FP64)
        h.sigma_device(z.data_ptr(), hz.data_ptr(), dg.FP64)
        w = 0.25 * x - 2.0 * z
        hw = torch.empty_like(x)
        h.sigma_device(w.data_ptr(), hw.data_ptr(), dg.FP64)
        torch.cuda.synchronize()
        a, b = float(torch.dot(z, hx)), float(torch.dot(x, hz))
        assert abs(a - b) <= 1e-12 * max(abs(a), 1.0) * 10
        lin = (hw - (0.25 * hx - 2.0 * hz)).abs().max().item()
        assert lin <= 1e-12 * hw.abs().max().item()
        xs = x.cpu().numpy()
        first = np.array([0, 17_000_000, D - 1000], dtype=np.uint64)
        length = np.array([1000, 1000, 1000], dtype=np.uint64)
        rows = np.concatenate([np.arange(f, f + n) for f, n in zip(first, length)]).astype(np.int64)
        dg_rows = h.diagonal()[rows]
        ref = o.gather_rows(xs, first, length, dg_rows)
        got = hx.cpu().numpy()[rows]
        assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("kernel", ["auto", "gather", "row1", "rowx", "pair", "tc"])
def test_sigma_L32_fp32_vs_oracle_samples(kernel, synth, dg):
    """L=32, N=16 (D = 601,080,390), FP32: sampled rank windows across the
    whole space (start, middle, end) against the FP64 oracle gather form."""
    torch = torch_cuda()
    p = synth(32, 16, 3)
    o = oracle.Ham(p, keep_diag=False)
    with dg.Hamiltonian.from_fcidump(p) as h:
        D = h.D
        h.set_sigma_kernel(kernel)
        g = torch.Generator(device="cuda").manual_seed(3)
        x = torch.randn(D, dtype=torch.float32, device="cuda", generator=g)
        y = torch.empty_like(x)
        h.sigma_device(x.data_ptr(), y.data_ptr(), dg.FP32)  # default stream: ordered after randn
        torch.cuda.synchronize()
        first = np.array([0, 12_870, 150_000_000, 300_540_000, 450_000_000, D - 20_000, D - 1000],
                         dtype=np.uint64)
        length = np.full(len(first), 1000, dtype=np.uint64)
        rows = np.concatenate([np.arange(f, f + n) for f, n in zip(first, length)]).astype(np.int64)
        xs = x.double().cpu().numpy()
        ref = o.gather_rows(xs, first, length, h.diagonal()[rows])
        got = y.cpu().numpy()[rows]
        err = np.abs(got - ref)
        bad = np.nonzero(err > 2e-6 * np.abs(ref).max())[0]
        assert bad.size == 0, (kernel, int(rows[bad[0]]), float(got[bad[0]]), float(ref[bad[0]]), int(bad.size))


@pytest.mark.parametrize("kernel", ["auto", "rowx", "gather", "rowff"])
def test_sigma_L32_fp64_vs_oracle_samples(kernel, synth, dg):
    """L=32, N=16 (D = 601,080,390), FP64 (the anchor and verification sigma
    of every mixed solve at this size): sampled rank windows across the whole
    space against the FP64 oracle gather form, 1e-12 of the largest |sigma|."""
    torch = torch_cuda()
    p = synth(32, 16, 3)
    o = oracle.Ham(p, keep_diag=False)
    with dg.Hamiltonian.from_fcidump(p) as h:
        D = h.D
        h.set_sigma_kernel(kernel)
        g = torch.Generator(device="cuda").manual_seed(11)
        x = torch.randn(D, dtype=torch.float64, device="cuda", generator=g)
        y = torch.empty_like(x)
        h.sigma_device(x.data_ptr(), y.data_ptr(), dg.FP64)
        torch.cuda.synchronize()
        first = np.array([0, 12_870, 150_000_000, 300_540_000, 450_000_000, D - 20_000, D - 1000],
                         dtype=np.uint64)
        length = np.full(len(first), 1000, dtype=np.uint64)
        rows = np.concatenate([np.arange(f, f + n) for f, n in zip(first, length)]).astype(np.int64)
        idx = torch.from_numpy(rows).cuda()
        xs = x.cpu().numpy()
        ref = o.gather_rows(xs, first, length, h.diagonal()[rows])
        got = y[idx].cpu().numpy()
        del x, y
        err = np.abs(got - ref)
        bad = np.nonzero(err > 1e-12 * np.abs(ref).max())[0]
        assert bad.size == 0, (kernel, int(rows[bad[0]]), float(got[bad[0]]), float(ref[bad[0]]), int(bad.size))


def test_default_stream_orders_after_caller_work(synth, dg):
    """A NULL stream is CUDA's default stream: a sigma queued right after the
    caller's own kernels on it sees their results (x written by randn)."""
    torch = torch_cuda()
    p = synth(28, 14, 2)
    with dg.Hamiltonian.from_fcidump(p) as h:
        outs = []
        for kernel in ("gather", "row1", "tc"):
            h.set_sigma_kernel(kernel)
            g = torch.Generator(device="cuda").manual_seed(9)
            x = torch.randn(h.D, dtype=torch.float32, device="cuda", generator=g)
            y = torch.empty_like(x)
            h.sigma_device(x.data_ptr(), y.data_ptr(), dg.FP32)
            outs.append(y)
        torch.cuda.synchronize()
        for o in outs[1:]:
            assert (outs[0] - o).abs().max().item() <= 2e-6 * outs[0].abs().max().item()


@pytest.mark.parametrize("kernel", ["auto", "gather", "row1"])
@pytest.mark.parametrize("L,N,seed,nv", [(16, 8, 41, 3), (20, 10, 42, 4), (12, 1, 43, 2), (24, 12, 44, 7),
                                         (18, 17, 45, 4), (26, 4, 46, 5)])
def test_sigma_block_vs_oracle(L, N, seed, nv, kernel, synth, dg):
    """doci_sigma_block: nv column-major vectors with padded leading
    dimensions against the oracle's matvec of each column (FP64 1e-12, FP32
    2e-6 of max|y|), and against doci_sigma column by column."""
    torch = torch_cuda()
    p = synth(L, N, seed)
    o = oracle.Ham(p)
    with dg.Hamiltonian.from_fcidump(p) as h:
        h.set_sigma_kernel(kernel)
        D = h.D
        ldx, ldy = D + 5, D + 3
        rng = np.random.default_rng(seed)
        X = rng.standard_normal((nv, D))
        refs = [o.matvec(X[v]) for v in range(nv)]
        for prec, dt, tol in ((dg.FP64, torch.float64, TOL64), (dg.FP32, torch.float32, TOL32)):
            xb = torch.zeros(nv * ldx, dtype=dt, device="cuda")
            for v in range(nv):
                xb[v * ldx:v * ldx + D] = torch.from_numpy(X[v]).to(dt)
            yb = torch.full((nv * ldy,), 7.0, dtype=dt, device="cuda")
            h.sigma_block_device(xb.data_ptr(), ldx, yb.data_ptr(), ldy, nv, prec)
            y1 = torch.empty(D, dtype=dt, device="cuda")
            torch.cuda.synchronize()
            for v in range(nv):
                y = yb[v * ldy:v * ldy + D].double().cpu().numpy()
                assert np.abs(y - refs[v]).max() <= tol * np.abs(refs[v]).max()
                if v < nv - 1:  # padding between columns untouched
                    assert bool((yb[v * ldy + D:(v + 1) * ldy] == 7.0).all())
                h.sigma_device(xb[v * ldx:].data_ptr(), y1.data_ptr(), prec)
                torch.cuda.synchronize()
                ys = y1.double().cpu().numpy()
                assert np.abs(y - ys).max() <= tol * np.abs(refs[v]).max()
                if kernel in ("gather", "row1"):  # same kernel family: same summation order
                    assert np.array_equal(y, ys)


def test_sigma_plan(synth, dg):
    """doci_sigma_plan reports the path doci_sigma takes: the automatic choice
    resolves to the mma.sync pair form for FP32 (a diag * x pass and the pair
    pass) and to the float-float pair form for FP64 (x conversion with the
    diag * x pass, and the pair pass) once the tiling gives every SM work (or
    to the shape's tuned choice), the gather kernel on small spaces; an explicit
    kind is honoured (the tensor-core pair form: one launch for the rows
    without column elements and one per row-part size of the (N-1)-pair sets,
    11 at L=20, N=10, split 9), FP32-only kinds take the automatic FP64 path,
    and the removed kinds are refused."""
    with dg.Hamiltonian.from_fcidump(synth(20, 10, 51)) as h:
        assert h.sigma_plan(dg.FP32) == (6, 2)
        auto64 = h.sigma_plan(dg.FP64)
        assert auto64 in ((9, 2), (1, 1), (3, 1), (4, 1))  # the float-float pair form, or a tuned choice
        h.set_sigma_kernel("row1")
        assert h.sigma_plan(dg.FP32) == (3, 1)
        h.set_sigma_kernel("pair")
        assert h.sigma_plan(dg.FP32) == (6, 2)
        assert h.sigma_plan(dg.FP64) == auto64  # FP32 only
        h.set_sigma_kernel("tc")
        assert h.sigma_plan(dg.FP32) == (8, 11)
        assert h.sigma_plan(dg.FP64) == auto64
        h.set_sigma_kernel("rowff")
        assert h.sigma_plan(dg.FP64) == (9, 2)
        assert h.sigma_plan(dg.FP32) == (6, 2)  # FP64 only
        for bad in (2, 5, 7, 10, -1):
            with pytest.raises(dg.DociError):
                h.set_sigma_kernel(bad)
    with dg.Hamiltonian.from_fcidump(synth(12, 6, 52)) as h:
        assert h.sigma_plan(dg.FP32) == (1, 1)
        assert h.sigma_plan(dg.FP64) == (1, 1)


@pytest.mark.parametrize("prec_name", ["FP64", "FP32"])
def test_sigma_host_pinned_and_pageable(prec_name, synth, dg):
    """doci_sigma_host on pinned host buffers (copied by kernels through
    their device mapping), on pageable ones (cudaMemcpyAsync), and on an
    offset inside a pinned buffer: all equal doci_sigma on device buffers."""
    torch = torch_cuda()
    import ctypes as C
    prec = getattr(dg, prec_name)
    tdt = torch.float64 if prec == dg.FP64 else torch.float32
    with dg.Hamiltonian.from_fcidump(synth(18, 9, 61)) as h:
        h.set_sigma_kernel("row1")  # deterministic: results compare bit for bit
        D = h.D
        x = torch.randn(D + 7, dtype=tdt, generator=torch.Generator().manual_seed(3))
        xd = x[:D].cuda()
        yd = torch.empty_like(xd)
        h.sigma_device(xd.data_ptr(), yd.data_ptr(), prec)
        torch.cuda.synchronize()
        ref = yd.cpu()
        lib = dg.lib()
        for pinned, off in ((True, 0), (True, 3), (False, 0)):
            xs = x.pin_memory() if pinned else x.clone()
            ys = torch.full((D + 7,), float("nan"), dtype=tdt)
            ys = ys.pin_memory() if pinned else ys
            src = xs[off:off + D] if off else xs[:D]
            if off:  # same values at an offset inside the buffer
                src.copy_(x[:D])
            st = lib.doci_sigma_host(h.handle, C.c_void_p(src.data_ptr()), C.c_void_p(ys[off:].data_ptr()), prec)
            assert st == 0
            assert torch.equal(ys[off:off + D], ref), (pinned, off)


@pytest.mark.parametrize("prec_name,kernel", [("FP32", "pair"), ("FP64", "rowff")])
@pytest.mark.parametrize("L,N,seed,off,pinned", [(22, 11, 31, 0, True), (24, 12, 30, 3, True), (20, 7, 33, 1, True),
                                                 (22, 11, 34, 0, False)])
def test_sigma_host_pair_overlapped_copies(prec_name, kernel, L, N, seed, off, pinned, synth, dg):
    """doci_sigma_host on the pair forms (FP32 kind 6, FP64-accurate kind 9)
    uploads x in pieces on a copy stream while the unit groups whose rows
    have all arrived run (each piece's diagonal pass before the first group
    reaching it) and downloads a pinned y piece by piece as no later group
    reaches it: the result matches the oracle within the precision's
    tolerance, for buffers at an offset and for pageable ones, and a second
    call on the same handle (reused stream, events, staging) agrees with the
    first."""
    torch = torch_cuda()
    import ctypes as C
    prec = getattr(dg, prec_name)
    tdt, tol = (torch.float32, TOL32) if prec == dg.FP32 else (torch.float64, TOL64)
    p = synth(L, N, seed)
    o = oracle.Ham(p)
    with dg.Hamiltonian.from_fcidump(p) as h:
        h.set_sigma_kernel(kernel)
        assert h.sigma_plan(prec)[0] == (6 if prec == dg.FP32 else 9)
        D = h.D
        x = np.random.default_rng(seed).standard_normal(D)
        yr = o.matvec(x)
        xs = torch.zeros(D + 8, dtype=tdt)
        ys = torch.full((D + 8,), float("nan"), dtype=tdt)
        if pinned:
            xs, ys = xs.pin_memory(), ys.pin_memory()
        xs[off:off + D] = torch.from_numpy(x).to(tdt)
        lib = dg.lib()
        outs = []
        for _ in range(2):
            st = lib.doci_sigma_host(h.handle, C.c_void_p(xs[off:].data_ptr()), C.c_void_p(ys[off:].data_ptr()), prec)
            assert st == 0
            outs.append(ys[off:off + D].numpy().astype(np.float64).copy())
        for y in outs:
            assert np.abs(y - yr).max() <= tol * np.abs(yr).max()
        assert np.abs(outs[0] - outs[1]).max() <= tol * np.abs(yr).max()


def test_autotune_keeps_parity(synth, dg):
    """doci_ham_autotune picks a path that fits, the plan reports it, sigma on
    the tuned path still matches the oracle, and a second handle of the same
    shape uses the same choice; block sigmas after tuning match too."""
    torch = torch_cuda()
    p = synth(20, 10, 71)
    o = oracle.Ham(p)
    with dg.Hamiltonian.from_fcidump(p) as h, dg.Hamiltonian.from_fcidump(synth(20, 10, 72)) as h2:
        for prec, tol in ((dg.FP32, TOL32), (dg.FP64, TOL64)):
            kind = h.autotune(prec, 1)
            assert kind in (1, 3, 4, 6)
            assert h.sigma_plan(prec)[0] == kind and h2.sigma_plan(prec)[0] == kind
            x = np.random.default_rng(7).standard_normal(h.D)
            yr = o.matvec(x)
            y = h.sigma(x.astype(np.float32) if prec == dg.FP32 else x, prec)
            assert np.abs(y - yr).max() <= tol * np.abs(yr).max()
            method = h.autotune(prec, 3)
            assert method in (1, 2, 3)
            tdt = torch.float64 if prec == dg.FP64 else torch.float32
            X = torch.from_numpy(np.random.default_rng(8).standard_normal((3, h.D))).to(tdt).cuda()
            Y = torch.empty_like(X)
            h.sigma_block_device(X.data_ptr(), h.D, Y.data_ptr(), h.D, 3, prec)
            torch.cuda.synchronize()
            for v in range(3):
                ref = o.matvec(X[v].double().cpu().numpy())
                assert np.abs(Y[v].double().cpu().numpy() - ref).max() <= tol * np.abs(ref).max()
