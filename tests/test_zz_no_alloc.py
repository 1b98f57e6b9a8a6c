"""doci_multidot_noalloc: the allocation-free variant of doci_multidot, for
callers that cannot let a library allocate device memory (their own
pre-reserved memory pool, or loops that cannot take an allocation's
synchronisation).  Called through the C ABI and compared with
doci_multidot on two calls in a row; the same tolerance as the FP64
reductions elsewhere (1e-12 relative).  Collected last (file name), and
self-contained so it also passes alone in a fresh process."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def lib():
    import doci_gb300
    L = doci_gb300.lib()
    vp, i, i64 = C.c_void_p, C.c_int, C.c_int64
    L.doci_multidot_noalloc.argtypes = [vp, i64, i, vp, i64, i, vp, vp]
    L.doci_multidot_noalloc.restype = i
    return L


@pytest.mark.parametrize("dtype,prec", [("float64", 0), ("float32", 1)])
def test_noalloc_matches_multidot_twice(lib, dtype, prec):
    import torch
    tdt = getattr(torch, dtype)
    n, m = 3_000_017, 19
    g = torch.Generator(device="cuda").manual_seed(11 + prec)
    V = torch.randn(m, n, dtype=tdt, device="cuda", generator=g)
    w = torch.randn(n, dtype=tdt, device="cuda", generator=g)
    ref = torch.empty(m, dtype=torch.float64, device="cuda")
    out = torch.full((m,), float("nan"), dtype=torch.float64, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())  # V, w, out were written on the default stream
    with torch.cuda.stream(s):
        assert lib.doci_multidot(C.c_void_p(V.data_ptr()), n, m, C.c_void_p(w.data_ptr()), n, prec,
                                 C.c_void_p(ref.data_ptr()), C.c_void_p(s.cuda_stream)) == 0
        for call in range(2):
            out.fill_(float("nan"))
            assert lib.doci_multidot_noalloc(C.c_void_p(V.data_ptr()), n, m, C.c_void_p(w.data_ptr()), n, prec,
                                             C.c_void_p(out.data_ptr()), C.c_void_p(s.cuda_stream)) == 0
            s.synchronize()
            r, o = ref.cpu().numpy(), out.cpu().numpy()
            assert np.all(np.isfinite(o)), call
            assert np.abs(o - r).max() <= TOL * np.abs(r).max(), call
    exact = (V.double() @ w.double()).cpu().numpy()
    assert np.abs(out.cpu().numpy() - exact).max() <= 1e-9 * np.abs(exact).max()


def test_noalloc_rejects_oversize_and_bad_args(lib):
    import torch
    V = torch.zeros(40, 8, dtype=torch.float64, device="cuda")
    w = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(40, dtype=torch.float64, device="cuda")
    st = lib.doci_multidot_noalloc(C.c_void_p(V.data_ptr()), 8, 33, C.c_void_p(w.data_ptr()), 8, 0,
                                   C.c_void_p(out.data_ptr()), None)
    assert st == 14  # DOCI_ERR_SCRATCH_LIMIT
    assert "scratch" in lib.doci_status_string(st).decode()
    assert lib.doci_multidot_noalloc(None, 8, 3, C.c_void_p(w.data_ptr()), 8, 0, C.c_void_p(out.data_ptr()),
                                     None) == 5  # DOCI_ERR_INVALID
