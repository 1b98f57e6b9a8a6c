"""CPU-side checks of the C ABI (no GPU needed): every symbol declared in
include/*.h is exported, the reference's own executable links against the
library, host-side input errors map to status codes, and the reader gives
bit-identical integrals to the oracle's."""
import ctypes as C
import os
import re
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, cuda_ok, reference_dir

HEADER = os.path.join(ROOT, "include", "doci_gb300.h")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b([A-Za-z_][A-Za-z0-9_]*)\s*\([^;{]*\)\s*;", src)
    return sorted({n for n in names if n not in ("void", "int", "matvec")})


@pytest.fixture(scope="module")
def lib():
    import doci_gb300
    return doci_gb300.lib()


def test_header_symbols_exported(lib):
    names = declared_functions()
    assert {"fill_doci_data", "doci_matvec", "sparse_eigensolve", "doci_sigma", "doci_solve"} <= set(names)
    out = subprocess.run(["nm", "-D", "--defined-only", lib._name], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (\w+)$", out, re.M))
    missing = [n for n in names if n not in exported]
    assert not missing, missing


@pytest.mark.skipif(not os.path.isdir(os.path.join(reference_dir(), "src")), reason="reference sources not present")
def test_reference_executable_links(lib, tmp_path):
    """The reference's executable.c + macros.c link against libdoci_gb300 in place of doci.c."""
    import glob
    import scipy
    ob = glob.glob(os.path.join(os.path.dirname(scipy.__file__), "..", "scipy.libs", "libscipy_openblas*.so"))
    if not ob:
        pytest.skip("no BLAS")
    R = reference_dir()
    exe = str(tmp_path / "doci_ref_on_gpu")
    pkg = os.path.join(ROOT, "doci_gb300")
    cmd = ["gcc", "-O2", "-Dnone=shared", f"-I{R}/include", "-Ddnrm2_=scipy_dnrm2_", "-Ddscal_=scipy_dscal_",
           f"{R}/src/executable.c", f"{R}/src/macros.c", "-L", pkg, "-ldoci_gb300", ob[0],
           f"-Wl,-rpath,{pkg}", f"-Wl,-rpath,{os.path.dirname(ob[0])}", "-lm", "-o", exe]
    subprocess.run(cmd, check=True)
    r = subprocess.run([exe, "--help"], capture_output=True, text=True)
    assert "DOCI" in r.stdout


def _status(lib, path):
    h = C.c_void_p()
    return lib.doci_ham_from_fcidump(path.encode(), C.byref(h))


def test_status_codes_without_gpu(lib, tmp_path, fcidump):
    bad = tmp_path / "bad.FCIDUMP"
    bad.write_text("not an fcidump\n")
    assert _status(lib, str(bad)) == 2  # DOCI_ERR_FORMAT
    assert _status(lib, str(tmp_path / "missing")) == 1  # DOCI_ERR_OPEN
    line = tmp_path / "line.FCIDUMP"
    line.write_text(" &FCI NORB=4,NELEC=4,MS2=0,\n &END\n 0.5 1 1 1 1\n garbage\n")
    assert _status(lib, str(line)) == 2
    oob = tmp_path / "oob.FCIDUMP"
    oob.write_text(" &FCI NORB=4,NELEC=4,MS2=0,\n &END\n 0.5 9 1 1 1\n")
    assert _status(lib, str(oob)) == 2
    big = tmp_path / "big.FCIDUMP"
    big.write_text(" &FCI NORB=33,NELEC=4,MS2=0,\n &END\n 0.5 1 1 1 1\n")
    assert _status(lib, str(big)) == 4  # DOCI_ERR_TOO_MANY_ORBITALS
    ms = tmp_path / "ms.FCIDUMP"
    ms.write_text(" &FCI NORB=4,NELEC=4,MS2=2,\n &END\n 0.5 1 1 1 1\n")
    assert _status(lib, str(ms)) == 3  # DOCI_ERR_NALPHA_NBETA
    if not cuda_ok():
        assert _status(lib, fcidump("H2O_STO3G")) == 8  # DOCI_ERR_NO_DEVICE
    assert lib.doci_status_string(3).decode().startswith("number of up and down")


def test_reader_matches_oracle(lib, fcidump):
    import oracle
    for name in ("H2O_STO3G", "H2O_631G", "synthetic_L10_N5_s3"):
        path = fcidump(name)
        L, Na, Nb = C.c_uint(), C.c_uint(), C.c_uint()
        core = C.c_double()
        one, two = C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
        lib.read_fcidump(path.encode(), C.byref(L), C.byref(Na), C.byref(Nb), C.byref(core), C.byref(one),
                         C.byref(two))
        n = L.value
        a1 = np.ctypeslib.as_array(one, (n * n,)).copy()
        a2 = np.ctypeslib.as_array(two, (n ** 4,)).copy()
        Lo, Nao, Nbo = C.c_uint(), C.c_uint(), C.c_uint()
        co = C.c_double()
        o1, o2 = C.POINTER(C.c_double)(), C.POINTER(C.c_double)()
        bad = C.c_int()
        assert oracle.lib().orc_read_fcidump(path.encode(), C.byref(Lo), C.byref(Nao), C.byref(Nbo), C.byref(co),
                                             C.byref(o1), C.byref(o2), C.byref(bad)) == 0
        assert (n, Na.value, Nb.value) == (Lo.value, Nao.value, Nbo.value)
        assert core.value == co.value
        assert np.array_equal(a1, np.ctypeslib.as_array(o1, (n * n,)))
        assert np.array_equal(a2, np.ctypeslib.as_array(o2, (n ** 4,)))


@pytest.mark.parametrize("content,msg", [
    (" &FCI NORB=4,NELEC=4,MS2=2,\n &END\n 0.5 1 1 1 1\n", "Number of up and down electrons not equal"),
    (" &FCI NORB=33,NELEC=4,MS2=0,\n &END\n 0.5 1 1 1 1\n", "Too many orbitals."),
    ("junk\n", "File is wrongly formatted."),
])
def test_fill_doci_data_fatal_errors_like_reference(content, msg, tmp_path):
    """fill_doci_data keeps the reference's fatal-error convention (message + exit)."""
    p = tmp_path / "f.FCIDUMP"
    p.write_text(content)
    code = (f"import sys; sys.path.insert(0, {ROOT!r}); import ctypes as C, doci_gb300; "
            f"L = doci_gb300.lib(); d = C.c_void_p(); L.fill_doci_data({str(p)!r}.encode(), C.byref(d))")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True)
    assert r.returncode == 1
    assert msg in r.stderr
