"""Writes the model panel of the multi-model batched workload.

Run in a container where the reference tree exists (its location in the
INFERNAL_REF_ROOT environment variable, or as the first argument):

    python tests/golden/gen_panel.py [reference_root]

Reads and configures (local mode, the CM file's QDB bands) the calibrated
CMs that ship with the reference (testsuite/*.c.cm, tutorial/*.c.cm) with the
project's reader (infernal_gb300/cmfile.py) and stores their score tables as
``panel/<name>.model.npz``.  The panel spans consensus lengths 71-307
(227-960 states, 0-7 bifurcations); tRNA, Vault and Plant_SRP are the golden
models one directory up, re-written here too so that every stored model
carries its CM file's E-value calibration lines (ECMLC/ECMGC/ECMLI/ECMGI).
"""
from __future__ import annotations

import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from infernal_gb300 import cmfile  # noqa: E402

PANEL = {"tRNA1415G": "testsuite", "snR75": "testsuite", "tRNA-Sec": "testsuite", "srp-euk": "testsuite",
         "rnaseP-eubact": "testsuite", "5S_rRNA": "tutorial", "Cobalamin": "tutorial", "tRNA5": "tutorial",
         "tRNA5-hand": "tutorial"}


def main(ref_root=None):
    ref_root = ref_root or os.environ.get("INFERNAL_REF_ROOT")
    if not ref_root:
        raise SystemExit("set INFERNAL_REF_ROOT (or pass the reference tree's location)")
    os.makedirs(os.path.join(HERE, "panel"), exist_ok=True)
    for name, sub in PANEL.items():
        m = cmfile.load(os.path.join(ref_root, sub, f"{name}.c.cm"))
        cmfile.save_npz(m, os.path.join(HERE, "panel", f"{name}.model.npz"))
        print(name, m.M, m.clen, m.W)
    for name in ("tRNA", "Vault", "Plant_SRP"):
        m = cmfile.load(os.path.join(ref_root, "testsuite", f"{name}.c.cm"))
        cmfile.save_npz(m, os.path.join(HERE, f"{name}.model.npz"))


if __name__ == "__main__":
    main(*sys.argv[1:])
