import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a); run with -m gpu")


@pytest.fixture(scope="session")
def golden():
    """(meta list, arrays) of tests/golden, produced by the reference's own scanners."""
    import json

    import numpy as np
    g = os.path.join(ROOT, "tests", "golden")
    with open(os.path.join(g, "golden.json")) as fh:
        meta = json.load(fh)
    arrays = dict(np.load(os.path.join(g, "golden.npz")))
    return meta, arrays


@pytest.fixture(scope="session")
def models():
    from infernal_gb300 import cmfile
    g = os.path.join(ROOT, "tests", "golden")
    return {n: cmfile.load_npz(os.path.join(g, f"{n}.model.npz")) for n in ("tRNA", "Vault", "Plant_SRP")}


def hits_from_golden(case):
    return [(h[0], h[1], h[2], h[3], float.fromhex(h[4])) for h in case["hits"]]
