"""The tensor-core sigma's bounded device waits (sigma_tc.cu).

In a child process whose wait limit is 0 (DOCI_TC_SPIN_LIMIT=0: every
mbarrier wait of the kernel gives up at once, as a wait on a barrier that
nothing completes would after its limit), doci_sigma_host must return
DOCI_ERR_DEVICE_TIMEOUT: the kernel sets its error word, drains its copies in
flight, frees its tensor memory and returns.  The context stays usable: a
sigma by another kernel in the same process afterwards matches the oracle.
No GPU fault, trap or endless wait is involved."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT

pytestmark = pytest.mark.gpu

CHILD = r"""
import ctypes as C, sys
import numpy as np
sys.path.insert(0, {root!r})
import doci_gb300 as dg, oracle
p = {path!r}
o = oracle.Ham(p)
with dg.Hamiltonian.from_fcidump(p) as h:
    h.set_sigma_kernel("tc")
    assert h.sigma_plan(dg.FP32)[0] == 8, h.sigma_plan(dg.FP32)
    x = np.random.default_rng(1).standard_normal(h.D).astype(np.float32)
    y = np.empty_like(x)
    st = dg.lib().doci_sigma_host(h.handle, x.ctypes.data_as(C.c_void_p), y.ctypes.data_as(C.c_void_p), dg.FP32)
    print("status", st)
    h.set_sigma_kernel("row1")
    y2 = h.sigma(x, dg.FP32)
    ref = o.matvec(x.astype(np.float64))
    print("after", float(np.abs(y2 - ref).max() / np.abs(ref).max()))
"""


def test_wait_limit_reports_timeout(synth):
    p = synth(20, 10, 71)
    env = dict(os.environ, DOCI_TC_SPIN_LIMIT="0")
    r = subprocess.run([sys.executable, "-c", CHILD.format(root=ROOT, path=p)], capture_output=True, text=True,
                       env=env, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = dict(ln.split(" ", 1) for ln in r.stdout.splitlines() if ln.startswith(("status", "after")))
    assert int(lines["status"]) == 12  # DOCI_ERR_DEVICE_TIMEOUT
    assert float(lines["after"]) <= 2e-6
