"""Stores the targets of the reference's known-answer sensitivity test.

Run in a container where the reference tree exists (its location in the
INFERNAL_REF_ROOT environment variable, or as the first argument):

    python tests/golden/gen_known_answers.py [reference_root]

testsuite/itest6-sensitivity.pl runs cmsearch with three calibrated CMs on
five test-suite sequences and checks the coordinates of the top hit.  This
script digitizes those sequences into ``known_answers.npz`` and writes the
cases (model, target, search options, expected top hit) to
``known_answers.json``; the models are in panel/ (gen_panel.py).  It also
stores the truncated-mode known answer of testsuite/itest7-trunc.pl (Vault on
tremitted-Vault.fa) in ``known_answers_trunc.json``.
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

# (model, target file, fbeta, beta, expected (sfrom, sto), line of the check in testsuite/itest6-sensitivity.pl)
CASES = [
    ("tRNA1415G", "mito-ascaris.fa", None, None, (4169, 4230), 112),
    ("srp-euk", "ffs-frag.fa", 1e-2, 1e-4, (15714, 15739), 150),
    ("srp-euk", "ffs-ecoli.fa", 1e-2, 1e-4, (43, 68), 158),
    ("rnaseP-eubact", "rnaseP-frag.fa", None, None, (10920, 10580), 196),
    ("rnaseP-eubact", "rnaseP-bsu.fa", None, None, (43, 383), 205),
]


# truncated mode (testsuite/itest7-trunc.pl:56-67): Vault on three truncated
# emitted sequences, default cmsearch -E 0.01: exactly two hits,
# (sequence, sfrom, sto, printed score)
TR_FILE = "tremitted-Vault.fa"
TR_HITS = [("Vault-1", 1, 63, 33.2), ("Vault-2", 1, 59, 25.5)]


def main(ref_root=None):
    ref_root = ref_root or os.environ.get("INFERNAL_REF_ROOT")
    if not ref_root:
        raise SystemExit("set INFERNAL_REF_ROOT (or pass the reference tree's location)")
    arrays, meta = {}, []
    for model, fa, fbeta, beta, (a, b), line in CASES:
        seq = cmfile.read_fasta(os.path.join(ref_root, "testsuite", fa))[0][1].upper().replace("T", "U")
        arrays["dsq." + fa] = cmfile.digitize(seq)
        meta.append(dict(model=model, target=fa, fbeta=fbeta, beta=beta, sfrom=a, sto=b,
                         source=f"testsuite/itest6-sensitivity.pl:{line}"))
    tr = cmfile.read_fasta(os.path.join(ref_root, "testsuite", TR_FILE))
    for name, seq in tr:
        arrays[f"trdsq.{name}"] = cmfile.digitize(seq.upper().replace("T", "U"))
    trunc = dict(model="Vault", target=TR_FILE, names=[n for n, _ in tr], E=0.01,
                 hits=[list(h) for h in TR_HITS], source="testsuite/itest7-trunc.pl:56-67")
    np.savez_compressed(os.path.join(HERE, "known_answers.npz"), **arrays)
    with open(os.path.join(HERE, "known_answers.json"), "w") as fh:
        json.dump(meta, fh, indent=1)
    with open(os.path.join(HERE, "known_answers_trunc.json"), "w") as fh:
        json.dump(trunc, fh, indent=1)


if __name__ == "__main__":
    main(*sys.argv[1:])
