"""The CPU restatement (oracle/cm_scan_oracle.c) against the golden vectors
written by the reference's own scanners (tests/golden/gen_golden.py)."""
import numpy as np
import pytest

import oracle
from conftest import hits_from_golden

# The restatement implements the Fast scanners' fold order; RefCYKScan gives
# the same CYK results (max is order-independent), RefIInsideScan does not.
ALGO = {"cyk": "cyk", "refcyk": "cyk", "inside": "inside", "finside": "finside"}


def _cases(golden):
    meta, _ = golden
    return [c for c in meta if c["algo"] in ALGO]


def test_golden_cases_present(golden):
    meta, arrays = golden
    assert len(meta) >= 50
    assert {c["model"] for c in meta} == {"tRNA", "Vault", "Plant_SRP"}
    assert {c["algo"] for c in meta} >= {"cyk", "inside", "refcyk", "refinside", "finside"}


@pytest.mark.parametrize("idx", range(0, 60))
def test_oracle_matches_reference(golden, models, idx):
    cases = _cases(golden)
    if idx >= len(cases):
        pytest.skip("no such case")
    c = cases[idx]
    _, arrays = golden
    m = models[c["model"]]
    dsq = arrays["dsq." + c["seq"]]
    hits, ei, ej, sc, vsc = oracle.scan(m, dsq, c["i0"], c["j0"], algo=ALGO[c["algo"]], qdbidx=c["qdbidx"],
                                        cutoff=c["cutoff"], do_null3=bool(c["null3"]), env_cutoff=c["env_cutoff"],
                                        notgreedy=bool(c["notgreedy"]))
    assert hits == hits_from_golden(c)
    assert (ei, ej) == (c["envi"], c["envj"])
    assert np.float32(sc) == np.float32(float.fromhex(c["sc"]))
    assert np.array_equal(vsc.view(np.int32), arrays[f"vsc.{c['id']}"].view(np.int32))


def test_ref_inside_order_differs_only_slightly(golden):
    """RefIInsideScan folds init first; its scores stay within a few
    thousandths of a bit of FastIInsideScan's (src/cm_dpsearch.c:2359)."""
    meta, _ = golden
    fast = {(c["model"], c["seq"]): c for c in meta if c["algo"] == "inside" and c["qdbidx"] == 2 and not c["notgreedy"]}
    n = 0
    for c in meta:
        if c["algo"] != "refinside":
            continue
        f = fast[(c["model"], c["seq"])]
        assert abs(float.fromhex(c["sc"]) - float.fromhex(f["sc"])) < 0.02
        n += 1
    assert n >= 3
