"""CPU check of the sigma kernels' neighbour-rank arithmetic: the device
enumeration code (addressing.cuh) compiled for the host and run over whole
small spaces and sampled large ones (every index in range and equal to the
direct lexical rank; every hop visited once)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "host_checks", "neighbours_check.cu")
ROW_SRC = os.path.join(HERE, "host_checks", "row_check.cu")
PAIR_SRC = os.path.join(HERE, "host_checks", "pair_check.cu")


@pytest.fixture(scope="module")
def exe(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("nb") / "neighbours_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", SRC, "-o", out], check=True)
    return out


@pytest.mark.parametrize("L,N,stride", [
    (1, 0, 1), (1, 1, 1), (4, 2, 1), (7, 3, 1), (10, 5, 1), (12, 1, 1), (12, 11, 1), (14, 7, 1),
    (16, 8, 1), (18, 5, 1), (20, 10, 7), (24, 12, 4099), (28, 14, 100003), (28, 7, 997), (32, 16, 1000003),
    (32, 1, 1), (32, 31, 1), (32, 2, 3), (32, 30, 3), (31, 15, 700001), (32, 0, 1), (32, 32, 1),
])
def test_neighbour_ranks(exe, L, N, stride):
    r = subprocess.run([exe, str(L), str(N), str(stride)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad=0" in r.stdout


@pytest.fixture(scope="module")
def row_exe(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("rowc") / "row_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", ROW_SRC, "-o", out], check=True)
    return out


@pytest.mark.parametrize("L,N,split,rs,cs", [
    (10, 5, 6, 1, 1), (12, 6, 8, 1, 1), (12, 3, 8, 1, 1), (12, 9, 8, 1, 1), (14, 7, 9, 1, 1),
    (16, 8, 10, 1, 1), (18, 9, 9, 1, 1), (20, 10, 9, 3, 5), (24, 12, 13, 7, 11), (28, 14, 16, 37, 101),
    (32, 16, 16, 257, 1009), (32, 2, 16, 1, 1), (32, 30, 16, 1, 1), (28, 7, 16, 5, 17), (9, 0, 8, 1, 1),
    (9, 9, 8, 1, 1), (17, 1, 16, 1, 1), (17, 16, 16, 1, 1),
    # the splits the library picks for small-N / large-N spaces (row part up to 24 orbitals)
    (32, 2, 8, 1, 1), (32, 30, 8, 1, 1), (32, 3, 8, 3, 1), (26, 4, 8, 1, 1), (24, 12, 13, 7, 11),
    (26, 4, 12, 1, 1), (22, 11, 11, 1, 7), (20, 10, 9, 1, 3),
])
def test_row_kernel_ranks(row_exe, L, N, split, rs, cs):
    r = subprocess.run([row_exe, str(L), str(N), str(split), str(rs), str(cs)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad=0" in r.stdout


@pytest.fixture(scope="module")
def pair_exe(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("pairc") / "pair_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-diag-suppress=20011", PAIR_SRC, "-o", out], check=True)
    return out


@pytest.mark.parametrize("L,N,split,bs,ss", [
    # whole spaces: every determinant reached once per pair it holds
    (10, 5, 6, 1, 1), (12, 6, 8, 1, 1), (12, 3, 8, 1, 1), (12, 11, 8, 1, 1), (14, 7, 9, 1, 1),
    (16, 8, 10, 1, 1), (18, 9, 9, 1, 1), (20, 10, 9, 1, 1), (9, 0, 8, 1, 1), (9, 9, 8, 1, 1),
    (17, 1, 16, 1, 1), (17, 16, 16, 1, 1), (32, 2, 8, 1, 1), (22, 11, 11, 1, 1),
    # sampled large spaces: every visited index in range and equal to the direct rank
    (32, 16, 16, 37, 101), (28, 14, 16, 11, 31), (32, 30, 8, 3, 1), (26, 4, 12, 1, 1), (24, 12, 13, 7, 11),
    (30, 15, 16, 29, 97), (31, 15, 16, 31, 101), (29, 14, 16, 13, 53), (27, 13, 15, 5, 23),
])
def test_pair_form_ranks(pair_exe, L, N, split, bs, ss):
    r = subprocess.run([pair_exe, str(L), str(N), str(split), str(bs), str(ss)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad=0" in r.stdout


TC_SRC = os.path.join(HERE, "host_checks", "tc_check.cu")


@pytest.fixture(scope="module")
def tc_exe(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("tcc") / "tc_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", TC_SRC, "-o", out], check=True)
    return out


@pytest.mark.parametrize("L,N,split,us,ss", [
    # whole spaces: every determinant reached once per pair it holds, its diagonal written once
    (10, 5, 6, 1, 1), (12, 6, 8, 1, 1), (12, 3, 8, 1, 1), (12, 11, 8, 1, 1), (14, 7, 9, 1, 1),
    (16, 8, 10, 1, 1), (18, 9, 9, 1, 1), (20, 10, 9, 1, 1), (9, 0, 8, 1, 1), (9, 9, 8, 1, 1),
    (17, 1, 16, 1, 1), (17, 16, 16, 1, 1), (22, 11, 11, 1, 1), (24, 12, 16, 1, 1), (6, 6, 6, 1, 1),
    (7, 0, 7, 1, 1), (32, 2, 16, 1, 1), (32, 30, 16, 1, 1),
    # sampled large spaces: every index in range and equal to the direct rank
    (32, 16, 16, 37, 101), (28, 14, 16, 11, 31), (30, 15, 16, 13, 7),
])
def test_tc_pair_form_ranks(tc_exe, L, N, split, us, ss):
    r = subprocess.run([tc_exe, str(L), str(N), str(split), str(us), str(ss)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad=0" in r.stdout


PLAN_SRC = os.path.join(HERE, "host_checks", "host_plan_check.cu")


@pytest.fixture(scope="module")
def plan_exe(tmp_path_factory):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not available")
    out = str(tmp_path_factory.mktemp("planc") / "host_plan_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-diag-suppress=20011", PLAN_SRC, "-o", out], check=True)
    return out


# the shapes' splits as the library picks them for a 152-SM GB300, plus edge shapes
PLAN_SHAPES = [(32, 16, 16), (31, 15, 16), (30, 15, 16), (29, 14, 16), (28, 14, 16), (27, 13, 15), (24, 12, 13),
               (22, 11, 11), (20, 10, 9), (18, 9, 9), (26, 4, 12), (32, 2, 8), (12, 6, 8), (17, 1, 16), (9, 9, 8)]


@pytest.mark.parametrize("L,N,split", PLAN_SHAPES)
def test_host_schedule_orders_copies_and_groups(plan_exe, L, N, split):
    """The host-buffer pair sigma's piece and group schedule (host_plan.h):
    every unit in one group within its pieces, and, in a happens-before
    simulation of the executor's three streams, each piece's upload and
    diagonal pass before every group reaching it and all of those before the
    piece's download."""
    r = subprocess.run([plan_exe, str(L), str(N), str(split)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad=0" in r.stdout


@pytest.mark.parametrize("plant", ["drop-up", "drop-other"])
def test_host_schedule_check_catches_planted_mistakes(plan_exe, plant):
    r = subprocess.run([plan_exe, "32", "16", "16", plant], capture_output=True, text=True)
    assert r.returncode == 1 and "bad=0" not in r.stdout, r.stdout + r.stderr
