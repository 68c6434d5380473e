"""Generates golden vectors for the model panel (tests/golden/panel).

Run in a container where the reference tree exists (its location in the
INFERNAL_REF_ROOT environment variable, or as the first argument):

    python tests/golden/gen_panel_golden.py [reference_root]

For each panel CM: a seeded 4.4 kb target (iid, 45% GC) with two sequences
sampled from the CM (infernal_gb300/emit.py) embedded on random strands,
scanned by the REFERENCE'S OWN FastCYKScan (QDB1, NULL3) and FastIInsideScan
(QDB2, NULL3), compiled from source by oracle/build_ref.sh.  Hits, envelope,
best score and per-state best scores go to ``golden_panel.npz`` /
``golden_panel.json``.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from infernal_gb300 import cmfile, emit  # noqa: E402
import oracle  # noqa: E402

PANEL = ["tRNA1415G", "snR75", "tRNA-Sec", "srp-euk", "rnaseP-eubact", "5S_rRNA", "Cobalamin", "tRNA5", "tRNA5-hand"]


def main(ref_root=None):
    ref_root = ref_root or oracle.reference_root()
    if not ref_root:
        raise SystemExit("set INFERNAL_REF_ROOT (or pass the reference tree's location)")
    if oracle.build_ref(ref_root) is None:
        raise SystemExit(f"reference tree not found under {ref_root}")
    rng = np.random.default_rng(20261207)
    arrays, meta = {}, []
    for name in PANEL:
        m = cmfile.load_npz(os.path.join(HERE, "panel", f"{name}.model.npz"))
        ins = [emit.sample(m, rng) for _ in range(2)]
        dsq, spans = emit.make_target(rng, 4400, 0.45, ins)     # one insert per 2 kb slot
        assert len(spans) == 2
        n = len(dsq) - 2
        arrays[f"dsq.{name}"] = dsq
        for algo, qdb in (("cyk", 1), ("inside", 2)):
            hits, ei, ej, sc, vsc = oracle.scan(m, dsq, 1, n, algo=algo, qdbidx=qdb, cutoff=0.0, do_null3=True,
                                                env_cutoff=2.0, reference=True)
            cid = len(meta)
            arrays[f"vsc.{cid}"] = vsc
            meta.append(dict(id=cid, model=name, seq=name, i0=1, j0=n, algo=algo, qdbidx=qdb, cutoff=0.0, null3=1,
                             env_cutoff=2.0, notgreedy=0, envi=ei, envj=ej, sc=float(np.float32(sc)).hex(),
                             hits=[[h[0], h[1], h[2], h[3], float(np.float32(h[4])).hex()] for h in hits]))
            print(f"{cid:3d} {name:14s} {algo:7s} qdb{qdb} hits={len(hits)} sc={sc:.3f}", flush=True)
    np.savez_compressed(os.path.join(HERE, "golden_panel.npz"), **arrays)
    with open(os.path.join(HERE, "golden_panel.json"), "w") as fh:
        json.dump(meta, fh, indent=0)


if __name__ == "__main__":
    main(*sys.argv[1:])
