"""The --nohmm search pipeline (infernal_gb300/pipeline.py): survivor-window
rules of pli_cyk_seq_filter, E-value arithmetic, and the reference's
known answers through the whole pipeline (CYK filter at F6, windows, final
Inside, E-values): the short SRP case on the CPU through the emulated
kernels, every case on the GPU."""
import json
import os

import numpy as np
import pytest

from infernal_gb300 import cmfile, lib as L, pipeline

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_cyk_windows_rules():
    W, L_ = 100, 10_000
    # hit (start, stop): window [stop - 99, start + 99]
    assert pipeline.cyk_windows([(500, 560)], W, L_) == [(461, 599)]
    # the second window (from its stop: 650 - 99 = 551) starts inside the first: merged, end from the second hit
    assert pipeline.cyk_windows([(600, 650), (500, 560)], W, L_) == [(461, 699)]
    # the second window starts after the first ends: apart
    assert pipeline.cyk_windows([(700, 760), (500, 560)], W, L_) == [(461, 599), (661, 799)]
    # adjacent but not overlapping windows stay apart
    assert pipeline.cyk_windows([(500, 560), (739, 800)], W, L_) == [(461, 599), (701, 838)]
    # clipped at the sequence ends
    assert pipeline.cyk_windows([(5, 40), (9960, 9990)], W, L_) == [(1, 104), (9891, 10_000)]


def _known():
    with open(os.path.join(HERE, "known_answers.json")) as fh:
        meta = json.load(fh)
    arrays = dict(np.load(os.path.join(HERE, "known_answers.npz")))
    return meta, arrays


def _model(c):
    m = cmfile.load_npz(os.path.join(HERE, "panel", f"{c['model']}.model.npz"))
    if c["fbeta"] is not None:
        d1, x1, d2, x2, _ = cmfile.qdb_bands(m, beta1=c["fbeta"], beta2=c["beta"], beta_W=1e-7)
        m.dmin1, m.dmax1, m.dmin2, m.dmax2 = d1, x1, d2, x2
    return m


# itest6-sensitivity.pl's E-value thresholds per model
E_OF = {"tRNA1415G": 1e-3, "srp-euk": 0.01, "rnaseP-eubact": 0.1}


def test_pipeline_known_answer_emulated(emu):
    meta, arrays = _known()
    c = [x for x in meta if x["target"] == "ffs-ecoli.fa"][0]
    m = _model(c)
    hits = pipeline.search(emu, m, [(c["target"], arrays["dsq." + c["target"]])], E=E_OF[c["model"]], toponly=True)
    assert hits and (hits[0].sfrom, hits[0].sto) == (c["sfrom"], c["sto"])
    assert hits[0].evalue <= E_OF[c["model"]] and hits[0].strand == "+"


@pytest.mark.gpu
def test_pipeline_known_answers_gpu():
    meta, arrays = _known()
    s = L.Scanner(0)
    try:
        for c in meta:
            m = _model(c)
            hits = pipeline.search(s, m, [(c["target"], arrays["dsq." + c["target"]])], E=E_OF[c["model"]])
            assert hits, c["source"]
            assert (hits[0].sfrom, hits[0].sto) == (c["sfrom"], c["sto"]), (c["source"], hits[:2])
    finally:
        s.close()


def _scan_models_case():
    from infernal_gb300 import emit
    ms = [cmfile.load_npz(os.path.join(HERE, f"{n}.model.npz")) for n in ("tRNA", "Vault")]
    rng = np.random.default_rng(44)
    s = emit.sample(ms[0], rng)
    seq = "".join(rng.choice(list("ACGU"), 20)) + s + "".join(rng.choice(list("ACGU"), 20))
    return ms, [("t1", cmfile.digitize(seq))]


def _per_model(scanner, ms, targets, E, toponly=False):
    out = []
    for t in targets:
        for a, m in enumerate(ms):
            out += [(a, h) for h in pipeline.search(scanner, m, [t], E=E, toponly=toponly)]
    return sorted(out, key=lambda x: (x[1].evalue, -x[1].score))


def test_scan_models_equals_per_model_search_emulated(emu):
    ms, targets = _scan_models_case()
    got = pipeline.scan_models(emu, ms, targets, E=10.0, toponly=True)
    want = _per_model(emu, ms, targets, 10.0, toponly=True)
    assert got == want and got


def test_scan_models_both_strands_emulated(emu):
    """Both strands: the emitted sequence sits on the minus strand, so its hit
    is found on the reverse complement and mapped back to top-strand
    coordinates (sfrom > sto), as the per-model search maps it."""
    from infernal_gb300 import emit
    ms, targets = _scan_models_case()
    name, d = targets[0]
    rc = [(name, emit.revcomp_dsq(d))]
    got = pipeline.scan_models(emu, ms, rc, E=10.0)
    want = _per_model(emu, ms, rc, 10.0)
    assert got == want and got
    assert any(h.strand == "-" and h.sfrom > h.sto for _, h in got)


@pytest.mark.gpu
def test_scan_models_equals_per_model_search_gpu():
    from infernal_gb300 import emit
    ms = [cmfile.load_npz(os.path.join(HERE, f"{n}.model.npz")) for n in ("tRNA", "Vault", "Plant_SRP")]
    rng = np.random.default_rng(45)
    targets = []
    for k in range(4):
        ins = [emit.sample(ms[k % 3], rng)]
        d, _ = emit.make_target(rng, 4000, 0.45, ins)
        targets.append((f"t{k}", d))
    s = L.Scanner(0)
    try:
        got = pipeline.scan_models(s, ms, targets, E=1.0)
        want = []
        for t in targets:
            lst = []
            for a, m in enumerate(ms):
                lst += [(a, h) for h in pipeline.search(s, m, [t], E=1.0)]
            want += sorted(lst, key=lambda x: (x[1].evalue, -x[1].score))
        assert got == want and len(got) >= 4
    finally:
        s.close()
