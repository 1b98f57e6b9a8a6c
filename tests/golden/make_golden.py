"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

    python tests/golden/make_golden.py [--ref /root/reference]

Needs the reference checkout (its tests/ FCIDUMPs and sources) and builds
oracle/_ref (the reference compiled from its own sources, oracle/Makefile).
Writes:
  molecules/<name>.FCIDUMP.gz   the reference's test integrals (tests/*.FCIDUMP),
                                gzipped, so GPU runs without the checkout can
                                use them;
  synthetic_L14_N7_s1.FCIDUMP   the CPU-runnable benchmark configuration
                                (L=14, N=7, seed 1) from doci_gb300.fcidump;
  synthetic_L10_N5_s3.FCIDUMP   a small synthetic case for CG;
  golden.json                   per case: L, N, D, reference energies and
                                iteration counts for SOLVER=D/CG/CGP from the
                                reference executable (-DDAVIDIT traces), the
                                full-precision Davidson energy, a checksum of
                                the reference diagonal and sigma of a seeded
                                vector (max-abs and 2-norm), and the published
                                values of tests/coHF.out and tests/lifHF.out;
  sigma_<case>.npz              for D <= 4000: x, reference sigma(x), diagonal,
                                and the reference bitstring table.
"""
from __future__ import annotations

import argparse
import ctypes as C
import gzip
import json
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from doci_gb300.fcidump import write_synthetic_fcidump  # noqa: E402

MOLECULES = ["H2O_STO3G", "N2_STO3G", "H2O_631G", "lili_321g", "lif_631g_1", "co_631g_1"]


def run_ref_exe(fcidump: str, solver: str, max_its: int, tol: float = 1e-8) -> dict:
    with tempfile.TemporaryDirectory() as td:
        inp = os.path.join(td, "in.in")
        with open(inp, "w") as f:
            f.write(f"FCIDUMP= {fcidump}\nSOLVER = {solver}\nMAX_ITS={max_its}\nTOL={tol:g}\nHF_INIT= 1\n")
        env = dict(os.environ, OMP_NUM_THREADS="4", OPENBLAS_NUM_THREADS="1")
        out = subprocess.run([oracle.REF_EXE_PATH, inp], capture_output=True, text=True, env=env, check=True).stdout
    rows = re.findall(r"^(\d+)\t(\d+)\t(\S+)\t(\S+)$", out, re.M)
    energy = float(re.search(r"\*\* DOCI ENERGY : (\S+)", out).group(1))
    code = int(re.search(r"\*\* EXIT CODE SOLVER : (\S+)", out).group(1))
    return {"energy_printed": energy, "exit_code": code,
            "trace": [[int(a), float(c), float(d)] for a, b, c, d in rows]}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default="/root/reference")
    a = ap.parse_args()
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={a.ref}", "all", "ref"], check=True)
    mol_dir = os.path.join(HERE, "molecules")
    os.makedirs(mol_dir, exist_ok=True)
    cases = {}
    work = tempfile.mkdtemp()
    for m in MOLECULES:
        src = os.path.join(a.ref, "tests", m + ".FCIDUMP")
        with open(src, "rb") as f, gzip.open(os.path.join(mol_dir, m + ".FCIDUMP.gz"), "wb", 9) as g:
            shutil.copyfileobj(f, g)
        cases[m] = src
    for name, (L, N, seed) in {"synthetic_L14_N7_s1": (14, 7, 1), "synthetic_L10_N5_s3": (10, 5, 3)}.items():
        p = os.path.join(HERE, name + ".FCIDUMP")
        write_synthetic_fcidump(p, L, N, seed)
        cases[name] = p
    R = oracle.ref_lib()
    golden = {"published": {
        "co_631g_1": {"energy": -112.8392190587, "iterations": 11, "source": "tests/coHF.out:39-43"},
        "lif_631g_1": {"energy": -107.0007150075, "iterations": 10, "source": "tests/lifHF.out:38-42"}},
        "cases": {}}
    for name, path in cases.items():
        rh = oracle.RefHam(path)
        D = rh.D
        L, N = R.ref_n_orbitals(rh._d), R.ref_n_pairs(rh._d)
        diag = rh.diag
        rng = np.random.default_rng(12345)
        x = rng.standard_normal(D)
        y = rh.matvec(x)
        # full-precision Davidson energy through the reference's own davidson()
        v = np.zeros(D)
        v[int(np.argmin(diag))] = 1.0
        e = C.c_double()
        d_ptr = R.doci_get_diagonal(rh._d)
        rc = R.davidson(v.ctypes.data_as(C.POINTER(C.c_double)), C.byref(e), 30, 2, 1e-8,
                        C.cast(R.doci_matvec, C.c_void_p), d_ptr, D, 1000, rh._d)
        entry = {"L": L, "N": N, "D": D, "diag_sum": float(diag.sum()), "diag_min": float(diag.min()),
                 "diag_argmin": int(np.argmin(diag)), "sigma_seed": 12345,
                 "sigma_maxabs": float(np.abs(y).max()), "sigma_norm": float(np.linalg.norm(y)),
                 "davidson": {"energy": e.value, "return_code": rc}}
        entry["D_exe"] = run_ref_exe(path, "D", 1000)
        if D <= 400000:
            entry["CG_exe"] = run_ref_exe(path, "CG", 60)
            entry["CGP_exe"] = run_ref_exe(path, "CGP", 60)
        golden["cases"][name] = entry
        if D <= 4000:
            np.savez_compressed(os.path.join(HERE, f"sigma_{name}.npz"), x=x, sigma=y, diag=diag,
                                bitstrings=rh.bitstrings)
        rh.close()
        print(name, L, N, D, entry["davidson"]["energy"], len(entry["D_exe"]["trace"]), flush=True)
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    shutil.rmtree(work, ignore_errors=True)


if __name__ == "__main__":
    main()
