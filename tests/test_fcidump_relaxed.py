"""The relaxed FCIDUMP reader: on canonically ordered files it gives the
reference reader's integrals exactly; on files with the same integrals in
any index order, shuffled lines, a multi-line namelist with other keys
(ORBSYM, ISYM), lower-case keys and Fortran D exponents it gives the same
canonical integrals; conflicting duplicates are a format error.  Host-only
(the reader runs on the CPU); the GPU test builds both Hamiltonians."""
import os
import random

import numpy as np
import pytest

MOLECULES = ["H2O_STO3G", "N2_STO3G", "H2O_631G", "lili_321g", "synthetic_L14_N7_s1", "synthetic_L10_N5_s3"]


def entries(path):
    """(value, i, j, k, l) lines and the header fields of an FCIDUMP."""
    with open(path) as f:
        lines = f.read().splitlines()
    head = lines[0]
    body = []
    started = False
    for ln in lines[1:]:
        if not started:
            t = ln.strip().upper()
            if t in ("&END", "/END", "/"):
                started = True
            continue
        if ln.strip():
            v, i, j, k, l = ln.split()
            body.append((v, int(i), int(j), int(k), int(l)))
    return head, body


def scramble(path, out, seed, dexp=True):
    """Same integrals: random one of the 8 index orders per entry, shuffled
    lines, the namelist spread over lines with ORBSYM/ISYM, lower-case keys."""
    import re
    head, body = entries(path)
    norb = int(re.search(r"NORB=\s*(\d+)", head).group(1))
    nelec = int(re.search(r"NELEC=\s*(\d+)", head).group(1))
    ms2 = int(re.search(r"MS2=\s*(-?\d+)", head).group(1))
    rng = random.Random(seed)
    rows = []
    for v, i, j, k, l in body:
        if k != 0:
            perms = [(i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                     (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)]
            i, j, k, l = rng.choice(perms)
        elif i != 0 and rng.random() < 0.5:
            i, j = j, i
        if dexp:
            v = v.replace("e", "D").replace("E", "D")
        rows.append(f"{v} {i} {j} {k} {l}")
    rng.shuffle(rows)
    with open(out, "w") as f:
        f.write(f" &fci norb = {norb},\n  nelec={nelec}, ms2 = {ms2},\n")
        f.write("  ORBSYM=" + ",".join("1" for _ in range(norb)) + ",\n  ISYM=1,\n &end\n\n")
        f.write("\n".join(rows) + "\n")


@pytest.fixture(scope="module")
def dg():
    import doci_gb300
    doci_gb300.lib()
    return doci_gb300


@pytest.mark.parametrize("name", MOLECULES)
def test_relaxed_equals_reference_on_canonical(name, fcidump, dg):
    p = fcidump(name)
    a = dg.fcidump_integrals(p, relaxed=False)
    b = dg.fcidump_integrals(p, relaxed=True)
    assert (a["L"], a["n_alpha"], a["n_beta"]) == (b["L"], b["n_alpha"], b["n_beta"])
    assert a["core"] == b["core"]
    assert np.array_equal(a["one"], b["one"]) and np.array_equal(a["two"], b["two"])


@pytest.mark.parametrize("name", MOLECULES)
@pytest.mark.parametrize("seed", [1, 2])
def test_relaxed_reads_any_order(name, seed, fcidump, dg, tmp_path):
    p = fcidump(name)
    q = str(tmp_path / f"{name}_{seed}.FCIDUMP")
    scramble(p, q, seed)
    a = dg.fcidump_integrals(p, relaxed=False)
    b = dg.fcidump_integrals(q, relaxed=True)
    assert (a["L"], a["n_alpha"], a["n_beta"], a["core"]) == (b["L"], b["n_alpha"], b["n_beta"], b["core"])
    assert np.array_equal(a["one"], b["one"]) and np.array_equal(a["two"], b["two"])


def test_reference_reader_loses_scrambled_entries(fcidump, dg, tmp_path):
    """What the relaxed reader fixes: the reference's reader cannot parse the
    multi-line header, and with its own header it drops non-canonical entries
    from the transform's domain."""
    p = fcidump("H2O_STO3G")
    q = str(tmp_path / "scr.FCIDUMP")
    scramble(p, q, 3, dexp=False)
    with pytest.raises(dg.DociError):
        dg.fcidump_integrals(q, relaxed=False)
    head, _ = entries(p)
    with open(q) as f:
        body = f.read().split("&end\n", 1)[1].lstrip("\n")  # the reference's reader takes no blank line
    r = str(tmp_path / "scr_head.FCIDUMP")
    with open(r, "w") as f:
        f.write(head + "\n &END\n" + body)
    a = dg.fcidump_integrals(p, relaxed=False)
    b = dg.fcidump_integrals(r, relaxed=False)
    assert not np.array_equal(a["two"], b["two"])


def test_relaxed_conflicting_duplicate(dg, tmp_path):
    q = str(tmp_path / "dup.FCIDUMP")
    with open(q, "w") as f:
        f.write("&FCI NORB=2,NELEC=2,MS2=0,\n&END\n 0.5 1 1 1 1\n 0.25 2 1 1 1\n 0.25 1 2 1 1\n"
                " 0.3 1 1 2 1\n -1.0 1 1 0 0\n -0.5 2 2 0 0\n 0.0 0 0 0 0\n")
    with pytest.raises(dg.DociError):
        dg.fcidump_integrals(q, relaxed=True)
    with open(q, "w") as f:
        f.write("&FCI NORB=2,NELEC=2,MS2=0,\n&END\n 0.5 1 1 1 1\n 0.25 2 1 1 1\n 0.25 1 2 1 1\n"
                " -1.0 1 1 0 0\n -0.5 2 2 0 0\n 0.0 0 0 0 0\n")
    b = dg.fcidump_integrals(q, relaxed=True)
    assert b["two"][1] == 0.25  # (21|11) at its canonical slot i=2, j=1, k=1, l=1


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["H2O_631G", "synthetic_L14_N7_s1"])
def test_relaxed_hamiltonian_on_gpu(name, fcidump, dg, tmp_path):
    p = fcidump(name)
    q = str(tmp_path / f"{name}.FCIDUMP")
    scramble(p, q, 7)
    with dg.Hamiltonian.from_fcidump(p) as a, dg.Hamiltonian.from_fcidump(q, relaxed=True) as b:
        assert a.D == b.D
        assert np.array_equal(a.diagonal(), b.diagonal())
        x = np.random.default_rng(1).standard_normal(a.D)
        assert np.array_equal(a.sigma(x, dg.FP64), b.sigma(x, dg.FP64))
