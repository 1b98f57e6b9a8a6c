import gzip
import json
import os
import shutil
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the sm_103a kernels)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def fcidump(tmp_path_factory):
    """fcidump(name) -> path of a golden FCIDUMP (molecules are decompressed)."""
    d = tmp_path_factory.mktemp("fcidump")

    def get(name: str) -> str:
        plain = os.path.join(GOLDEN, name + ".FCIDUMP")
        if os.path.exists(plain):
            return plain
        out = str(d / (name + ".FCIDUMP"))
        if not os.path.exists(out):
            with gzip.open(os.path.join(GOLDEN, "molecules", name + ".FCIDUMP.gz"), "rb") as f, open(out, "wb") as g:
                shutil.copyfileobj(f, g)
        return out

    return get


@pytest.fixture(scope="session")
def synth(tmp_path_factory):
    """synth(L, N, seed) -> path of a synthetic FCIDUMP (generated once)."""
    from doci_gb300.fcidump import write_synthetic_fcidump
    d = tmp_path_factory.mktemp("synth")

    def get(L: int, N: int, seed: int) -> str:
        p = str(d / f"s_L{L}_N{N}_{seed}.FCIDUMP")
        if not os.path.exists(p):
            write_synthetic_fcidump(p, L, N, seed)
        return p

    return get


def reference_dir() -> str:
    """The reference checkout ($DOCI_REFERENCE, else `reference` beside the
    repository); tests that read it skip where it is absent."""
    return os.environ.get("DOCI_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")


def cuda_ok() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False
