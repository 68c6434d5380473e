"""One scan of a stored model on a seeded synthetic target, for profiling.

    python -m infernal_gb300.profile_case <model> <length> <cyk|inside> [tile_rows arena]

<model> is a configured model under tests/golden (tRNA, Vault, Plant_SRP).
Runs the scan twice (the first builds the plan) and prints the kernel time.
With tile_rows/arena the launch shape is fixed (arena 1 shared, 2 global);
without them the autotuner picks it first.
"""
from __future__ import annotations

import os
import sys
import time

import numpy as np

from . import cmfile, emit, lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def main(argv):
    name = argv[1] if len(argv) > 1 else "Plant_SRP"
    L = int(argv[2]) if len(argv) > 2 else 30000
    algo = argv[3] if len(argv) > 3 else "cyk"
    q = 1 if algo == "cyk" else 2
    m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", f"{name}.model.npz"))
    dsq, _ = emit.make_target(np.random.default_rng(1), L, 0.40, [])
    sc = lib.Scanner(0)
    if len(argv) > 5:
        sc.set_shape(int(argv[4]), 0, 0, 0, int(argv[5]))
        shape = (int(argv[4]), int(argv[5]))
    else:
        shape = sc.autotune(m, q, algo)
    for _ in range(2):
        t = time.time()
        r = sc.scan(m, dsq, 1, L, algo=algo, qdbidx=q, cutoff=10.0)
        print(f"{name} L={L} {algo} shape={shape} kernel_ms={r.kernel_ms:.2f} wall_s={time.time() - t:.2f} hits={len(r.hits)}")
    sc.close()


if __name__ == "__main__":
    main(sys.argv)
