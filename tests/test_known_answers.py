"""The reference's known-answer sensitivity test (testsuite/itest6-sensitivity.pl):
the top hit of three calibrated CMs on five test-suite sequences, searched
on both strands, must start and end where the test says.

The scans are the final Inside stage as cmsearch runs it: FastIInsideScan
at the QDB2 bands, local mode, NULL3, greedy resolution.  srp-euk runs with
its bands recalculated at --fbeta 1e-2 / --beta 1e-4 (cmsearch.c
configure_cm: the QDBs are recomputed when the betas differ from the file's;
W stays the file's).  The reference's default pipeline (tRNA1415G,
rnaseP-eubact) filters with HMMs first and its final stage uses HMM bands;
its top hits are the QDB scan's top hits too.  CPU: the oracle over a 3 kb
window around each expected hit on its strand (whole targets take minutes on
one core); GPU: whole targets, both strands, every case."""
import json
import os

import numpy as np
import pytest

import oracle
from infernal_gb300 import cmfile, emit, lib as L

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _cases():
    with open(os.path.join(HERE, "known_answers.json")) as fh:
        meta = json.load(fh)
    arrays = dict(np.load(os.path.join(HERE, "known_answers.npz")))
    return meta, arrays


def _model(c):
    m = cmfile.load_npz(os.path.join(HERE, "panel", f"{c['model']}.model.npz"))
    if c["fbeta"] is not None:
        d1, x1, d2, x2, W = cmfile.qdb_bands(m, beta1=c["fbeta"], beta2=c["beta"], beta_W=1e-7)
        assert W == m.W                     # beta_W unchanged: the file's W
        m.dmin1, m.dmax1, m.dmin2, m.dmax2 = d1, x1, d2, x2
    return m


def _strand_coords(h, L, strand):
    return (h[0], h[1]) if strand == "+" else (L - h[0] + 1, L - h[1] + 1)


def test_known_answer_cases_present():
    meta, arrays = _cases()
    assert len(meta) == 5 and all("dsq." + c["target"] in arrays for c in meta)


@pytest.mark.parametrize("k", range(5))
def test_known_answer_top_hit_oracle(k):
    meta, arrays = _cases()
    c = meta[k]
    m = _model(c)
    dsq = arrays["dsq." + c["target"]]
    n = len(dsq) - 2
    plus = c["sfrom"] <= c["sto"]
    d = dsq if plus else emit.revcomp_dsq(dsq)
    a, b = (c["sfrom"], c["sto"]) if plus else (n - c["sfrom"] + 1, n - c["sto"] + 1)
    i0, j0 = max(1, a - 1500), min(n, b + 1500)
    hits = oracle.scan(m, d, i0, j0, algo="inside", qdbidx=2, cutoff=0.0, env_cutoff=0.0)[0]
    top = max(hits, key=lambda h: h[4])
    assert _strand_coords(top, n, "+" if plus else "-") == (c["sfrom"], c["sto"]), (c["source"], top)


@pytest.mark.gpu
def test_known_answer_top_hits_gpu():
    meta, arrays = _cases()
    s = L.Scanner(0)
    try:
        for c in meta:
            m = _model(c)
            dsq = arrays["dsq." + c["target"]]
            n = len(dsq) - 2
            best = []
            for strand, d in (("+", dsq), ("-", emit.revcomp_dsq(dsq))):
                r = s.scan(m, d, 1, n, algo="inside", qdbidx=2, cutoff=0.0, env_cutoff=0.0)
                best += [(h[4],) + _strand_coords(h, n, strand) for h in r.hits]
            top = max(best)
            assert top[1:] == (c["sfrom"], c["sto"]), (c["source"], top)
    finally:
        s.close()
