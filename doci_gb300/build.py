"""Build libdoci_gb300.so (sm_103a) and the `doci` executable in-tree.

    python -m doci_gb300.build            # library + executable
    python -m doci_gb300.build --clean

Every translation unit under doci_gb300/csrc is compiled by nvcc for
sm_103a only (``-gencode arch=compute_103a,code=sm_103a``), in parallel, into
doci_gb300/_build/, then linked with the static CUDA runtime into
doci_gb300/libdoci_gb300.so.  The `doci` command-line program
(csrc/doci_main.c) links against that library.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libdoci_gb300.so")
EXE = os.path.join(PKG, "doci")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3", "-I", os.path.join(ROOT, "include")]


def _sources():
    out = []
    for f in sorted(os.listdir(CSRC)):
        if f.endswith((".cu", ".cpp")):
            out.append(os.path.join(CSRC, f))
    return out


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [NVCC, *ARCH, *COMMON, "-c", src, "-o", obj]
    if os.environ.get("DOCI_PTXAS_VERBOSE") and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip() and os.environ.get("DOCI_PTXAS_VERBOSE"):
        print(r.stderr, file=sys.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    main_c = os.path.join(PKG, "cli", "doci_main.c")
    if os.path.exists(main_c):
        cmd = ["gcc", "-O2", "-std=gnu11", "-I", os.path.join(ROOT, "include"), main_c, "-o", EXE,
               "-L", PKG, "-ldoci_gb300", "-Wl,-rpath,$ORIGIN", "-lm"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"doci executable failed to build:\n{r.stdout}\n{r.stderr}")
    return LIB


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)
    for p in (LIB, EXE):
        if os.path.exists(p):
            os.remove(p)


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--clean", action="store_true")
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    if a.clean:
        clean()
    else:
        print(build(a.verbose))
