"""Generates the golden vectors of the scan parity tests.

Run in a container where the reference tree exists (its location in the
INFERNAL_REF_ROOT environment variable, or as the first argument):

    python tests/golden/gen_golden.py [reference_root]

It (1) reads and configures three of the reference test-suite CMs with the
project's reader (infernal_gb300/cmfile.py) and stores their score tables as
``<name>.model.npz``; (2) builds seeded target sequences -- iid background
with the reference test suite's CM-emitted sequences (testsuite/emitted-*.fa)
embedded on both strands, plus short, sub-range and degenerate-residue cases;
(3) runs the REFERENCE'S OWN scanners (FastCYKScan, RefCYKScan,
FastIInsideScan, RefIInsideScan, FastFInsideScan; src/cm_dpsearch.c, and the
truncated RefTrCYKScan / RefITrInsideScan of src/cm_dpsearch_trunc.c on
5'/3'-truncated targets for pipeline passes 2-5; compiled from source by
oracle/build_ref.sh) on every case and stores hits, envelope, best score (and
mode), and per-state best scores in ``golden.npz`` / ``golden.json``.

The parity tests replay these cases against the CPU restatement
(oracle/cm_scan_oracle.c) and against the GPU scanners.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from infernal_gb300 import cmfile  # noqa: E402
import oracle  # noqa: E402

MODELS = {"tRNA": "emitted-tRNA.fa", "Vault": "emitted-Vault.fa", "Plant_SRP": "tremitted-Plant_SRP.fa"}
COMP = str.maketrans("ACGU", "UGCA")


def revcomp(s: str) -> str:
    return s.translate(COMP)[::-1]


def make_target(rng, L, gc, inserts):
    """iid background of length L with the given strings embedded at
    non-overlapping random positions, each on a random strand."""
    p = [(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2]
    bg = list(rng.choice(list("ACGU"), L, p=p))
    pos = sorted(rng.choice(np.arange(0, L - 600), size=len(inserts), replace=False))
    out, last = [], 0
    for k, (ps, ins) in enumerate(zip(pos, inserts)):
        ps = max(ps, last)
        s = ins if rng.random() < 0.5 else revcomp(ins)
        out.append("".join(bg[last:ps]))
        out.append(s)
        last = ps
    out.append("".join(bg[last:]))
    return "".join(out)[: L + sum(len(x) for x in inserts)]


def cases_for(name, rng, emitted):
    """(label, sequence, i0, j0) cases of one model."""
    cs = []
    seq = make_target(rng, 2400, 0.5, emitted)
    cs.append(("emb", seq, 1, len(seq)))
    cs.append(("sub", seq, 37, len(seq) - 50))
    short = emitted[0][: max(20, len(emitted[0]) // 2)]
    cs.append(("short", short, 1, len(short)))
    deg = list(make_target(rng, 700, 0.4, emitted[:1]))
    for k in rng.choice(len(deg), 12, replace=False):
        deg[k] = rng.choice(list("NRYHBVDKMSW"))
    deg = "".join(deg)
    cs.append(("degen", deg, 1, len(deg)))
    return cs


def tr_cases_for(name, rng, emitted):
    """Truncated-scan cases: a 5'-truncated emitted sequence at the start of
    the target and a 3'-truncated one at its end, as the pipeline's terminal
    windows see them."""
    s = emitted[1 % len(emitted)]
    bg = lambda n: "".join(rng.choice(list("ACGU"), n))
    c5 = int(rng.integers(len(s) // 5, len(s) // 2))
    c3 = int(rng.integers(len(s) // 2, 4 * len(s) // 5))
    t5 = s[c5:] + bg(int(len(s) * 0.8))
    t3 = bg(int(len(s) * 0.7)) + s[:c3]
    return [("tr5", t5, 1, len(t5)), ("tr3", t3, 1, len(t3)), ("tr3sub", t3, 9, len(t3))]


TR_RUNS = [  # (algo, qdbidx, pass_idx, cutoff, null3, env_cutoff, notgreedy, which cases)
    ("trcyk", 1, 2, 0.0, 1, 2.0, 0, "all"),
    ("trcyk", 1, 3, 0.0, 1, 2.0, 0, "all"),
    ("trcyk", 1, 4, 0.0, 1, 2.0, 0, "all"),
    ("trcyk", 0, 4, -5.0, 0, 0.0, 0, "tr5"),
    ("trcyk", 2, 5, 0.0, 1, 2.0, 0, "tr3"),
    ("trcyk", 1, 4, 0.0, 1, 2.0, 1, "tr5"),
    ("trinside", 2, 2, 0.0, 1, 2.0, 0, "all"),
    ("trinside", 2, 3, 0.0, 1, 2.0, 0, "all"),
    ("trinside", 2, 4, 0.0, 1, 2.0, 0, "all"),
    ("trinside", 1, 4, 3.0, 0, 0.0, 1, "tr3"),
]


RUNS = [  # (algo, qdbidx, cutoff, null3, env_cutoff, notgreedy, which cases)
    ("cyk", 1, 0.0, 1, 2.0, 0, "all"),
    ("cyk", 2, 0.0, 0, 5.0, 0, "all"),
    ("cyk", 0, -5.0, 1, 0.0, 0, "short"),
    ("refcyk", 1, 0.0, 1, 2.0, 0, "emb"),
    ("cyk", 1, 0.0, 1, 2.0, 1, "emb"),
    ("inside", 2, 0.0, 1, 2.0, 0, "all"),
    ("inside", 1, 3.0, 0, 0.0, 0, "emb"),
    ("inside", 2, 0.0, 1, 2.0, 1, "emb"),
    ("refinside", 2, 0.0, 1, 2.0, 0, "emb"),
    ("finside", 2, 0.0, 1, 2.0, 0, "emb"),
]


def main(ref_root=None):
    ref_root = ref_root or oracle.reference_root()
    if not ref_root:
        raise SystemExit("set INFERNAL_REF_ROOT (or pass the reference tree's location)")
    so = oracle.build_ref(ref_root)
    if so is None:
        raise SystemExit(f"reference tree not found under {ref_root}")
    rng = np.random.default_rng(20261203)
    arrays, meta = {}, []
    for name, fa in MODELS.items():
        m = cmfile.load(os.path.join(ref_root, "testsuite", f"{name}.c.cm"))
        cmfile.save_npz(m, os.path.join(HERE, f"{name}.model.npz"))
        emitted = [s.upper().replace("T", "U") for _, s in cmfile.read_fasta(os.path.join(ref_root, "testsuite", fa))]
        for label, seq, i0, j0 in cases_for(name, rng, emitted):
            key = f"{name}.{label}"
            dsq = cmfile.digitize(seq)
            arrays[f"dsq.{key}"] = dsq
            for algo, qdb, cut, n3, envc, ng, which in RUNS:
                if which != "all" and which != label:
                    continue
                hits, ei, ej, sc, vsc = oracle.scan(m, dsq, i0, j0, algo=algo, qdbidx=qdb, cutoff=cut,
                                                    do_null3=bool(n3), env_cutoff=envc, notgreedy=bool(ng),
                                                    reference=True)
                cid = len(meta)
                arrays[f"vsc.{cid}"] = vsc
                meta.append(dict(id=cid, model=name, seq=key, i0=i0, j0=j0, algo=algo, qdbidx=qdb, cutoff=cut,
                                 null3=n3, env_cutoff=envc, notgreedy=ng, envi=ei, envj=ej,
                                 sc=float(np.float32(sc)).hex(),
                                 hits=[[h[0], h[1], h[2], h[3], float(np.float32(h[4])).hex()] for h in hits]))
                print(f"{cid:3d} {key:18s} {algo:9s} qdb{qdb} n3={n3} ng={ng} hits={len(hits)} sc={sc:.3f}")
    # truncated scanners (RefTrCYKScan / RefITrInsideScan), own seeded stream
    rng = np.random.default_rng(20261204)
    for name, fa in MODELS.items():
        m = cmfile.load_npz(os.path.join(HERE, f"{name}.model.npz"))
        emitted = [s.upper().replace("T", "U") for _, s in cmfile.read_fasta(os.path.join(ref_root, "testsuite", fa))]
        for label, seq, i0, j0 in tr_cases_for(name, rng, emitted):
            key = f"{name}.{label}"
            dsq = cmfile.digitize(seq)
            arrays[f"dsq.{key}"] = dsq
            for algo, qdb, pidx, cut, n3, envc, ng, which in TR_RUNS:
                if which != "all" and which != label:
                    continue
                hits, ei, ej, sc, vsc, mode = oracle.tr_scan(m, dsq, i0, j0, algo=algo, qdbidx=qdb, pass_idx=pidx,
                                                             cutoff=cut, do_null3=bool(n3), env_cutoff=envc,
                                                             notgreedy=bool(ng), reference=True)
                cid = len(meta)
                arrays[f"vsc.{cid}"] = vsc
                meta.append(dict(id=cid, model=name, seq=key, i0=i0, j0=j0, algo=algo, qdbidx=qdb, pass_idx=pidx,
                                 cutoff=cut, null3=n3, env_cutoff=envc, notgreedy=ng, envi=ei, envj=ej,
                                 sc=float(np.float32(sc)).hex(), mode=mode,
                                 hits=[[h[0], h[1], h[2], h[3], float(np.float32(h[4])).hex()] for h in hits]))
                print(f"{cid:3d} {key:18s} {algo:9s} qdb{qdb} pass{pidx} n3={n3} ng={ng} hits={len(hits)} sc={sc:.3f} mode={mode}")
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **arrays)
    with open(os.path.join(HERE, "golden.json"), "w") as fh:
        json.dump(meta, fh, indent=0)


if __name__ == "__main__":
    main(*sys.argv[1:])
