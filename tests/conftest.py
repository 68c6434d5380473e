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


@pytest.fixture(scope="session")
def emu():
    """The C ABI built for the test-only host-thread emulation of a CTA
    (g++, CMGB_HOST_EMULATION): the kernel source runs on CPU threads."""
    import subprocess
    from infernal_gb300 import lib as L
    so = os.path.join(ROOT, "tests", "emu", "_build", "libinfernal_gb300_emu.so")
    os.makedirs(os.path.dirname(so), exist_ok=True)
    csrc = os.path.join(ROOT, "infernal_gb300", "csrc")
    srcs = [os.path.join(csrc, f) for f in ("capi.cu", "filter.cu", "scan_plan.cpp", "hits.cpp", "calibrate.cpp")]
    deps = [os.path.join(csrc, f) for f in os.listdir(csrc)] + [os.path.join(ROOT, "include", "infernal_gb300.h"),
                                                             os.path.join(ROOT, "tests", "emu", "cmgb_emu.h")]
    if not os.path.exists(so) or os.path.getmtime(so) < max(os.path.getmtime(s) for s in deps):
        tmp = so + f".tmp{os.getpid()}"
        subprocess.check_call(["g++", "-std=c++20", "-O2", "-fPIC", "-shared", "-ffp-contract=off",
                               "-DCMGB_HOST_EMULATION", "-I", os.path.join(ROOT, "tests", "emu"),
                               "-x", "c++", srcs[0], srcs[1], "-x", "none", srcs[2], srcs[3], srcs[4], "-o", tmp, "-lpthread"])
        os.replace(tmp, so)
    return L.Scanner(lib=L.bind(so))
