"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
import os
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("oracle", "pi-bem_gb300"):
    p = os.path.join(REPO, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def oracle_mod():
    subprocess.run(["make", "-s", "-C", os.path.join(REPO, "oracle"), "oracle"], check=True)
    import oracle

    return oracle


@pytest.fixture(scope="session")
def pibem_mod():
    import pibem

    return pibem


@pytest.fixture(scope="session")
def synthetic():
    import synthetic

    return synthetic


def reference_dir():
    """The reference checkout, where this machine has one: $PIBEM_REFERENCE, else
    the directory the oracle's recipe compiled the reference classes from
    (oracle/_ref/reference_dir.txt); None when neither exists."""
    d = os.environ.get("PIBEM_REFERENCE")
    if not d:
        rec = os.path.join(REPO, "oracle", "_ref", "reference_dir.txt")
        if os.path.exists(rec):
            with open(rec) as f:
                d = f.read().strip()
    return d if d and os.path.isdir(d) else None


def rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))
