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
one core); GPU: whole targets, both strands, every case.

Truncated mode (testsuite/itest7-trunc.pl): Vault on three truncated
emitted reads must give exactly two hits with E <= 0.01, at the reference's
coordinates; the oracle and the GPU run the truncated Inside scanner over
passes 2-4 and both strands, and the emulated kernel matches the oracle on
the reads and passes that report the hits."""
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


def _trunc_hits(scan):
    """Per read: the best hit with E <= 0.01 over both strands and the
    truncated passes 2, 3 and 4 (5' only, 3' only, 5' and 3'), as the
    default pipeline runs them on reads that are terminal at both ends."""
    with open(os.path.join(HERE, "known_answers_trunc.json")) as fh:
        c = json.load(fh)
    _, arrays = _cases()
    m = cmfile.load_npz(os.path.join(HERE, f"{c['model']}.model.npz"))
    reads = [arrays["trdsq." + n] for n in c["names"]]
    Z = 2 * sum(len(d) - 2 for d in reads)
    li = m.ecm["ECMLI"]
    found = []
    for name, dsq in zip(c["names"], reads):
        n = len(dsq) - 2
        best = None
        for strand, d in (("+", dsq), ("-", emit.revcomp_dsq(dsq))):
            for p in (2, 3, 4):
                for h in scan(m, d, n, p):
                    if L.evalue(li, h[4], Z) <= c["E"] and (best is None or h[4] > best[3]):
                        best = (name,) + _strand_coords(h, n, strand) + (h[4],)
        if best:
            found.append(best)
    return c, found


def _check_trunc(c, found):
    # exactly the reference's hits; scores within 0.15 bits of the printed
    # one-decimal scores (the reference's default pipeline scores truncated
    # hits with HMM-banded Inside, these are QDB-banded: 33.10 vs 33.2,
    # 25.46 vs 25.5)
    assert [f[:3] for f in found] == [tuple(h[:3]) for h in c["hits"]], found
    for f, h in zip(found, c["hits"]):
        assert abs(f[3] - h[3]) < 0.15, (f, h)


def test_known_answer_truncated_oracle():
    c, found = _trunc_hits(lambda m, d, n, p: oracle.tr_scan(m, d, 1, n, algo="trinside", qdbidx=2, pass_idx=p,
                                                             cutoff=0.0, env_cutoff=0.0)[0])
    _check_trunc(c, found)


def test_known_answer_truncated_emulated(emu):
    """The emulated truncated kernel gives the oracle's hit list, bit for bit,
    on the two reads that hold the known hits, at the passes that report
    them (5'-truncated for Vault-1, 3'-truncated for Vault-2)."""
    _, arrays = _cases()
    m = cmfile.load_npz(os.path.join(HERE, "Vault.model.npz"))
    for name, p in (("Vault-1", 2), ("Vault-2", 3)):
        d = arrays["trdsq." + name]
        n = len(d) - 2
        r = emu.tr_scan(m, d, 1, n, algo="trinside", qdbidx=2, pass_idx=p, cutoff=0.0, env_cutoff=0.0)
        o = oracle.tr_scan(m, d, 1, n, algo="trinside", qdbidx=2, pass_idx=p, cutoff=0.0, env_cutoff=0.0)
        assert r.hits == o[0] and r.hits, name


@pytest.mark.gpu
def test_known_answer_truncated_gpu():
    s = L.Scanner(0)
    try:
        c, found = _trunc_hits(lambda m, d, n, p: s.tr_scan(m, d, 1, n, algo="trinside", qdbidx=2, pass_idx=p,
                                                            cutoff=0.0, env_cutoff=0.0).hits)
    finally:
        s.close()
    _check_trunc(c, found)
