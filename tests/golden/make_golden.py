"""Regenerate the golden fixtures in tests/golden/ from the reference itself.

    python tests/golden/make_golden.py --ref <reference checkout>   (or $DOCI_REFERENCE)
    python tests/golden/make_golden.py --ref <...> --l28 [--threads T]

Needs the reference checkout (its tests/ FCIDUMPs and sources) and builds
oracle/_ref (the reference compiled from its own sources, oracle/Makefile).
--exe only (re)makes exe/*.out: the reference executable's stdout
(EXE_CASES below), built with and without -DDAVIDIT, run on one thread.
--l28 only (re)makes the entry "synthetic_L28_N14_s2" of golden.json:
the reference executable's Davidson (DAVIDSON_MAX_VEC 30, DAVIDSON_KEEP 2,
TOL 1e-8, HF start) and CGP (MAX_ITS 40) runs on the seeded L=28, N=14
Hamiltonian (D = 40,116,600), with their iteration traces and wall times on
T OpenMP threads (several minutes of CPU; about 20 GB of host memory).
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
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from doci_gb300.fcidump import write_synthetic_fcidump  # noqa: E402

MOLECULES = ["H2O_STO3G", "N2_STO3G", "H2O_631G", "lili_321g", "lif_631g_1", "co_631g_1"]


def run_ref_exe(fcidump: str, solver: str, max_its: int, tol: float = 1e-8, threads: int = 4,
                extra: str = "", timed: bool = False) -> dict:
    with tempfile.TemporaryDirectory() as td:
        inp = os.path.join(td, "in.in")
        with open(inp, "w") as f:
            f.write(f"FCIDUMP= {fcidump}\nSOLVER = {solver}\nMAX_ITS={max_its}\nTOL={tol:g}\nHF_INIT= 1\n{extra}")
        env = dict(os.environ, OMP_NUM_THREADS=str(threads), OPENBLAS_NUM_THREADS="1")
        t0 = time.perf_counter()
        out = subprocess.run([oracle.REF_EXE_PATH, inp], capture_output=True, text=True, env=env, check=True).stdout
        wall = time.perf_counter() - t0
    rows = re.findall(r"^(\d+)\t(\d+)\t(\S+)\t(\S+)$", out, re.M)
    energy = float(re.search(r"\*\* DOCI ENERGY : (\S+)", out).group(1))
    code = int(re.search(r"\*\* EXIT CODE SOLVER : (\S+)", out).group(1))
    r = {"energy_printed": energy, "exit_code": code,
         "trace": [[int(a), float(c), float(d)] for a, b, c, d in rows]}
    if timed:
        r["wall_s"] = round(wall, 2)
        r["threads"] = threads
    return r


# name, molecule, input keys (besides FCIDUMP); the input echo names the
# FCIDUMP by the relative path "<molecule>.FCIDUMP"
EXE_CASES = [
    ("H2O_631G_D", "H2O_631G", "SOLVER = D\nTOL = 1e-8\nHF_INIT = 1\n"),
    ("H2O_631G_CGP", "H2O_631G", "SOLVER = CGP\nMAX_ITS = 60\nTOL = 1e-8\n"),
    ("lif_631g_1_D", "lif_631g_1", "SOLVER = D\nMAX_ITS = 100\nTOL = 1e-8\nDAVIDSON_KEEP = 2\n"
                                   "DAVIDSON_MAX_VEC = 30\nHF_INIT = 1\n"),
    ("co_631g_1_D", "co_631g_1", "SOLVER = D\nTOL = 1e-8\nDAVIDSON_MAX_VEC = 12\nDAVIDSON_KEEP = 3\n"),
]


def exe_outputs(ref: str) -> None:
    out_dir = os.path.join(HERE, "exe")
    os.makedirs(out_dir, exist_ok=True)
    env = dict(os.environ, OMP_NUM_THREADS="1", OPENBLAS_NUM_THREADS="1")
    for name, mol, keys in EXE_CASES:
        with tempfile.TemporaryDirectory() as td:
            shutil.copy(os.path.join(ref, "tests", mol + ".FCIDUMP"), os.path.join(td, mol + ".FCIDUMP"))
            with open(os.path.join(td, "in.in"), "w") as f:
                f.write(f"FCIDUMP = {mol}.FCIDUMP\n{keys}")
            for exe, tag in ((oracle.REF_EXE_PATH, "davidit"), (oracle.REF_EXE_PLAIN_PATH, "plain")):
                r = subprocess.run([exe, "in.in"], capture_output=True, text=True, env=env, cwd=td, check=True)
                with open(os.path.join(out_dir, f"{name}.{tag}.out"), "w") as f:
                    f.write(r.stdout)
        print(name, flush=True)


def l28_entry(ref: str, threads: int) -> None:
    """The plain FP64 Davidson and CGP of the L=28, N=14 Hamiltonian (seed 2)
    through the reference executable; merged into golden.json."""
    L, N, seed = 28, 14, 2
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, f"synthetic_L{L}_N{N}_s{seed}.FCIDUMP")
        write_synthetic_fcidump(p, L, N, seed)
        dav = run_ref_exe(p, "D", 1000, threads=threads, extra="DAVIDSON_KEEP = 2\nDAVIDSON_MAX_VEC = 30\n",
                          timed=True)
        print("D", dav["energy_printed"], len(dav["trace"]), dav["wall_s"], flush=True)
        cgp = run_ref_exe(p, "CGP", 40, threads=threads, timed=True)
        print("CGP", cgp["energy_printed"], len(cgp["trace"]), cgp["wall_s"], flush=True)
    gp = os.path.join(HERE, "golden.json")
    with open(gp) as f:
        golden = json.load(f)
    golden["cases"][f"synthetic_L{L}_N{N}_s{seed}"] = {
        "L": L, "N": N, "D": 40116600, "seed": seed, "generated": "doci_gb300.fcidump.write_synthetic_fcidump",
        "D_exe": dav, "CGP_exe": cgp,
        "settings": {"D": "DAVIDSON_MAX_VEC 30, DAVIDSON_KEEP 2, TOL 1e-8, HF_INIT 1, MAX_ITS 1000",
                     "CGP": "TOL 1e-8, HF_INIT 1, MAX_ITS 40"},
        "host": f"{os.cpu_count()} cores ({threads} OpenMP threads), OPENBLAS_NUM_THREADS=1"}
    with open(gp, "w") as f:
        json.dump(golden, f, indent=1)


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("DOCI_REFERENCE"),
                    help="reference checkout (default: $DOCI_REFERENCE)")
    ap.add_argument("--l28", action="store_true", help="only the L=28, N=14 entry")
    ap.add_argument("--exe", action="store_true", help="only the executable's stdout fixtures")
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 4)
    a = ap.parse_args()
    if not a.ref:
        ap.error("give --ref or set DOCI_REFERENCE")
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), f"REF={a.ref}", "all", "ref"], check=True)
    if a.l28:
        l28_entry(a.ref, a.threads)
        return
    if a.exe:
        exe_outputs(a.ref)
        return
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
