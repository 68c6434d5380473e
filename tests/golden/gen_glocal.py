"""Generates the golden vectors of the glocal-mode scan parity tests.

Run in a container where the reference tree exists (its location in the
INFERNAL_REF_ROOT environment variable, or as the first argument):

    python tests/golden/gen_glocal.py [reference_root]

It reads the three golden CMs with the project's reader configured in glocal
mode (no local begins or ends, cm_Configure without cm_localize; cmsearch -g)
and stores them as ``<name>.glocal.model.npz``; builds seeded targets with
the reference test suite's emitted sequences embedded (as gen_golden.py
does, own seeded stream); runs the REFERENCE'S OWN scanners (FastCYKScan,
FastIInsideScan, FastFInsideScan, compiled from source by
oracle/build_ref.sh) on every case and stores hits, envelope, best score and
per-state best scores in ``golden_glocal.npz`` / ``golden_glocal.json``.
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

from infernal_gb300 import cmfile  # noqa: E402
import oracle  # noqa: E402
from gen_golden import MODELS, make_target  # noqa: E402

RUNS = [  # (algo, qdbidx, cutoff, null3, env_cutoff, which cases)
    ("cyk", 1, 0.0, 1, 2.0, "all"),
    ("cyk", 2, -5.0, 0, 0.0, "emb"),
    ("inside", 2, 0.0, 1, 2.0, "all"),
    ("finside", 2, 0.0, 1, 2.0, "emb"),
]


def main(ref_root=None):
    ref_root = ref_root or oracle.reference_root()
    if not ref_root:
        raise SystemExit("set INFERNAL_REF_ROOT (or pass the reference tree's location)")
    so = oracle.build_ref(ref_root)
    if so is None:
        raise SystemExit(f"reference tree not found under {ref_root}")
    rng = np.random.default_rng(20261206)
    arrays, meta = {}, []
    for name, fa in MODELS.items():
        m = cmfile.load(os.path.join(ref_root, "testsuite", f"{name}.c.cm"), local=False)
        cmfile.save_npz(m, os.path.join(HERE, f"{name}.glocal.model.npz"))
        emitted = [s.upper().replace("T", "U") for _, s in cmfile.read_fasta(os.path.join(ref_root, "testsuite", fa))]
        seq = make_target(rng, 1500, 0.5, emitted[:3])
        short = emitted[0]
        for label, s, i0, j0 in (("emb", seq, 1, len(seq)), ("short", short, 1, len(short))):
            key = f"{name}.{label}"
            dsq = cmfile.digitize(s)
            arrays[f"dsq.{key}"] = dsq
            for algo, qdb, cut, n3, envc, which in RUNS:
                if which != "all" and which != label:
                    continue
                hits, ei, ej, sc, vsc = oracle.scan(m, dsq, i0, j0, algo=algo, qdbidx=qdb, cutoff=cut,
                                                    do_null3=bool(n3), env_cutoff=envc, reference=True)
                cid = len(meta)
                arrays[f"vsc.{cid}"] = vsc
                meta.append(dict(id=cid, model=name, seq=key, i0=i0, j0=j0, algo=algo, qdbidx=qdb, cutoff=cut,
                                 null3=n3, env_cutoff=envc, notgreedy=0, envi=ei, envj=ej,
                                 sc=float(np.float32(sc)).hex(),
                                 hits=[[h[0], h[1], h[2], h[3], float(np.float32(h[4])).hex()] for h in hits]))
                print(f"{cid:3d} {key:18s} {algo:9s} qdb{qdb} n3={n3} hits={len(hits)} sc={sc:.3f}")
    np.savez_compressed(os.path.join(HERE, "golden_glocal.npz"), **arrays)
    with open(os.path.join(HERE, "golden_glocal.json"), "w") as fh:
        json.dump(meta, fh, indent=0)


if __name__ == "__main__":
    main(*sys.argv[1:])
