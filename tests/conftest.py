import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

KAT_PATH = os.path.join(ROOT, "tests", "golden", "mrg8_kat.json")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and libmrg8g.so")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def oracle():
    from oracle.pyoracle import Oracle
    return Oracle()


@pytest.fixture(scope="session")
def kat():
    with open(KAT_PATH) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def reflib():
    """The reference compiled from its own sources (only where it exists)."""
    from oracle.pyoracle import REF_DIR, RefLib, reference_dir
    refdir = reference_dir()
    if refdir is None:
        pytest.skip("reference sources not found: set MRG8_REFERENCE or build them with "
                    "make -C oracle ref REF=<dir>")
    if not os.path.exists(os.path.join(REF_DIR, "libmrg8_ref_original.so")):
        import subprocess
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={refdir}"], check=True)
    return {f: RefLib(f, refdir) for f in RefLib.FLAVOURS}


@pytest.fixture(scope="session")
def lib():
    """libmrg8g.so, built in-tree if needed (no CPU fallback)."""
    import mrg8_gb300
    from mrg8_gb300 import build
    build.build()
    return mrg8_gb300.load()


@pytest.fixture(scope="session")
def cuda(lib):
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.init()
    return torch.device("cuda:0")


def u32(a):
    return np.asarray(a, dtype=np.uint32)
