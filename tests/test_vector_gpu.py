"""doci_multidot (the Davidson projection / subspace-column reduction) on
device buffers: FP64 accumulation, deterministic, both storage types."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("m", [1, 7, 16, 32])
@pytest.mark.parametrize("dtype,prec", [("float64", 0), ("float32", 1)])
def test_multidot(m, dtype, prec):
    import torch
    import doci_gb300
    L = doci_gb300.lib()
    tdt = getattr(torch, dtype)
    n, ld = 1_000_003, 1_000_011
    g = torch.Generator(device="cuda").manual_seed(m + 100 * prec)
    V = torch.randn(m, ld, dtype=tdt, device="cuda", generator=g)
    w = torch.randn(n, dtype=tdt, device="cuda", generator=g)
    out = torch.empty(m, dtype=torch.float64, device="cuda")
    out2 = torch.empty_like(out)
    for o in (out, out2):
        assert L.doci_multidot(C.c_void_p(V.data_ptr()), ld, m, C.c_void_p(w.data_ptr()), n, prec,
                               C.c_void_p(o.data_ptr()), None) == 0
    torch.cuda.synchronize()
    exact = (V[:, :n].double() @ w.double()).cpu().numpy()
    got = out.cpu().numpy()
    scale = V[:, :n].abs().max().item() * w.abs().max().item()
    assert np.abs(got - exact).max() <= 1e-12 * np.sqrt(n) * scale
    assert np.array_equal(got, out2.cpu().numpy())  # fixed reduction order


def test_multidot_invalid():
    import doci_gb300
    L = doci_gb300.lib()
    assert L.doci_multidot(None, 10, 3, None, 10, 0, None, None) == 5
