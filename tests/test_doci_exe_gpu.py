"""The `doci` executable against the reference executable's own stdout.

tests/golden/exe/*.out are the reference program's stdout (src/executable.c
with doci.c, davidson.c, CG.c), built with and without -DDAVIDIT, on the
reference's test molecules (made by tests/golden/make_golden.py --exe).  The
GPU program runs the same input file; every line must be identical except:

* wall-clock times (elapsed time, average time per matvec, ELAPSED TIME);
* the banner's executor line (doci.c:122-131 prints the OpenMP thread
  count; here the GPU is named);
* per-iteration numbers: the iteration number and INFO exactly, the energy
  (printed %f) within one unit of its last digit, the residue (printed %e)
  within 1e-4 relative or 1e-13 absolute, because GPU and CPU sum the
  vectors in different orders; d_energy (a difference of nearly equal
  energies, 1e-14 at convergence) is not compared.

The -DDAVIDIT table is switched on in the GPU program by DOCI_DAVIDIT=1.
"""
import gzip
import os
import re
import shutil
import subprocess

import pytest

from conftest import GOLDEN, ROOT, cuda_ok

EXE = os.path.join(ROOT, "doci_gb300", "doci")
CASES = [("H2O_631G_D", "H2O_631G", "SOLVER = D\nTOL = 1e-8\nHF_INIT = 1\n"),
         ("H2O_631G_CGP", "H2O_631G", "SOLVER = CGP\nMAX_ITS = 60\nTOL = 1e-8\n"),
         ("lif_631g_1_D", "lif_631g_1", "SOLVER = D\nMAX_ITS = 100\nTOL = 1e-8\nDAVIDSON_KEEP = 2\n"
                                        "DAVIDSON_MAX_VEC = 30\nHF_INIT = 1\n"),
         ("co_631g_1_D", "co_631g_1", "SOLVER = D\nTOL = 1e-8\nDAVIDSON_MAX_VEC = 12\nDAVIDSON_KEEP = 3\n")]

TIME_LINE = re.compile(r"^(elapsed time : |average time per matvec : |\t\t \*\* ELAPSED TIME : )")
ROW = re.compile(r"^(\d+)\t(-?\d+)\t(\S+)\t(\S+)$")
CONV = re.compile(r"^(Davidson|CG) converged in (\d+) iterations with (\S+) residue and d_energy (\S+)\.$")


def _close(a: str, b: str, rel: float, abs_: float) -> bool:
    fa, fb = float(a), float(b)
    return abs(fa - fb) <= max(abs_, rel * max(abs(fa), abs(fb)))


def compare(ours: str, ref: str):
    a, b = ours.splitlines(), ref.splitlines()
    assert len(a) == len(b), f"{len(a)} lines vs the reference's {len(b)}:\n{ours}"
    for la, lb in zip(a, b):
        if TIME_LINE.match(lb):
            assert TIME_LINE.match(la), (la, lb)
            continue
        if lb.startswith("\t** executing DOCI ("):
            assert la.startswith("\t** executing DOCI ("), (la, lb)
            continue
        ma, mb = ROW.match(la), ROW.match(lb)
        if mb:
            assert ma, (la, lb)
            assert ma.group(1) == mb.group(1) and ma.group(2) == mb.group(2), (la, lb)
            assert _close(ma.group(3), mb.group(3), 1e-4, 1e-13), (la, lb)
            assert abs(float(ma.group(4)) - float(mb.group(4))) <= 1.01e-6, (la, lb)
            continue
        ma, mb = CONV.match(la), CONV.match(lb)
        if mb:
            assert ma and ma.group(1) == mb.group(1) and ma.group(2) == mb.group(2), (la, lb)
            assert _close(ma.group(3), mb.group(3), 1e-4, 1e-13), (la, lb)
            continue
        assert la == lb, (la, lb)


@pytest.mark.gpu
@pytest.mark.skipif(not cuda_ok(), reason="needs a GPU")
@pytest.mark.parametrize("variant", ["plain", "davidit"])
@pytest.mark.parametrize("name,mol,keys", CASES, ids=[c[0] for c in CASES])
def test_doci_executable_stdout(tmp_path, name, mol, keys, variant):
    assert os.path.exists(EXE), "doci executable not built (doci_gb300.build)"
    with gzip.open(os.path.join(GOLDEN, "molecules", mol + ".FCIDUMP.gz"), "rb") as f, \
            open(tmp_path / (mol + ".FCIDUMP"), "wb") as g:
        shutil.copyfileobj(f, g)
    (tmp_path / "in.in").write_text(f"FCIDUMP = {mol}.FCIDUMP\n{keys}")
    env = dict(os.environ)
    env.pop("DOCI_DAVIDIT", None)
    env.pop("DOCI_MIXED", None)
    if variant == "davidit":
        env["DOCI_DAVIDIT"] = "1"
    r = subprocess.run([EXE, "in.in"], capture_output=True, text=True, cwd=tmp_path, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    with open(os.path.join(GOLDEN, "exe", f"{name}.{variant}.out")) as f:
        ref = f.read()
    compare(r.stdout, ref)


def test_compare_rules_on_reference_pairs():
    """The comparison itself (CPU): each fixture matches itself, a changed
    energy digit, iteration count or echo line is caught, timings are not."""
    with open(os.path.join(GOLDEN, "exe", "H2O_631G_D.davidit.out")) as f:
        ref = f.read()
    compare(ref, ref)
    compare(ref.replace("elapsed time : ", "elapsed time : 9").replace("ELAPSED TIME : ", "ELAPSED TIME : 7"), ref)
    for bad in (ref.replace("DOCI ENERGY : -76.0125161011", "DOCI ENERGY : -76.0125161012"),
                ref.replace("converged in 9 iterations", "converged in 10 iterations"),
                ref.replace("TOL              = 1.000000e-08", "TOL              = 1.000000e-07"),
                ref.replace("-76.012516\n", "-76.012519\n", 1)):
        with pytest.raises(AssertionError):
            compare(bad, ref)
