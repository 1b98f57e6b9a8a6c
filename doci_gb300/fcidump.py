"""Seeded synthetic FCIDUMP files for the DOCI workloads.

Integral model (the benchmark configurations' generator):
  * h symmetric, h_ii uniform in [-2, 0.5] sorted ascending, h_ij ~ N(0, 0.05);
  * (ij|kl) = sum_{P=1}^{2L} B^P_ij B^P_kl with B^P symmetric, upper-triangle
    entries ~ N(0, 0.1) -- 8-fold symmetric with K_ia = (ia|ia) >= 0;
  * E_core = 0, NELEC = 2N, MS2 = 0.
Lines are written "%.17e i j k l", 1-based, in canonical order (i >= j,
k >= l, ij >= kl), the only order the reader's symmetrisation propagates
from (src/doci.c:640-655).
"""
from __future__ import annotations

import numpy as np


def synthetic_integrals(L: int, seed: int):
    """(h, eri) of the synthetic model; eri[i, j, k, l] = (ij|kl), 0-based."""
    rng = np.random.default_rng(seed)
    h = rng.normal(0.0, 0.05, (L, L))
    h = np.triu(h, 1)
    h = h + h.T
    h[np.diag_indices(L)] = np.sort(rng.uniform(-2.0, 0.5, L))
    B = rng.normal(0.0, 0.1, (2 * L, L, L))
    B = np.triu(B)
    B = B + np.transpose(B, (0, 2, 1)) - np.einsum("pii->pi", B)[:, :, None] * np.eye(L)
    eri = np.einsum("pij,pkl->ijkl", B, B, optimize=True)
    return h, eri


def write_fcidump(path: str, h: np.ndarray, eri: np.ndarray, n_pairs: int, core: float = 0.0) -> None:
    L = h.shape[0]
    lines = [" &FCI NORB=%d,NELEC=%d,MS2=0,\n" % (L, 2 * n_pairs), "  ORBSYM=%s\n" % ("1," * L),
             "  ISYM=1,\n", " &END\n"]
    ii, jj = np.tril_indices(L)          # i >= j, row-major over i
    pair = ii * (ii + 1) // 2 + jj
    for a in range(len(ii)):
        i, j = ii[a], jj[a]
        sel = pair <= pair[a]
        ks, ls = ii[sel], jj[sel]
        vals = eri[i, j, ks, ls]
        lines.extend("%.17e %d %d %d %d\n" % (v, i + 1, j + 1, k + 1, l + 1)
                     for v, k, l in zip(vals.tolist(), ks.tolist(), ls.tolist()))
    for i, j in zip(ii.tolist(), jj.tolist()):
        lines.append("%.17e %d %d 0 0\n" % (h[i, j], i + 1, j + 1))
    lines.append("%.17e 0 0 0 0\n" % core)
    with open(path, "w") as f:
        f.writelines(lines)


def write_synthetic_fcidump(path: str, L: int, n_pairs: int, seed: int) -> str:
    h, eri = synthetic_integrals(L, seed)
    write_fcidump(path, h, eri, n_pairs)
    return path


def raw_integrals(L: int, seed: int):
    """The synthetic integrals in the layout read_fcidump produces for the
    canonical file (only canonical entries set; the transform mirrors them):
    one[i + j L] and two[i + j L + k L^2 + l L^3]."""
    h, eri = synthetic_integrals(L, seed)
    one = np.zeros((L, L))
    two = np.zeros((L, L, L, L))
    ii, jj = np.tril_indices(L)
    one[jj, ii] = h[ii, jj]  # file line "h i j 0 0" lands at one[(j-1) L + (i-1)]
    pair = ii * (ii + 1) // 2 + jj
    for a in range(len(ii)):
        sel = pair <= pair[a]
        ks, ls = ii[sel], jj[sel]
        two[ls, ks, jj[a], ii[a]] = eri[ii[a], jj[a], ks, ls]
    # memory order: index i fastest -> C-order array indexed [l, k, j, i]
    return one.reshape(-1), two.reshape(-1)
