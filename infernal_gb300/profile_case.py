"""One scan of a stored model on a seeded synthetic target, for profiling.

    python -m infernal_gb300.profile_case <model> <length> <cyk|inside|finside> [tile_rows arena [ctas_per_sm]]
    python -m infernal_gb300.profile_case <model> <nreads> <trcyk|trinside> [tile_rows arena [ctas_per_sm]]
    python -m infernal_gb300.profile_case <model> <length> filter
    python -m infernal_gb300.profile_case <model> <length> learned


<model> is a configured model under tests/golden (tRNA, Vault, Plant_SRP).
The standard scanners scan one target of <length> residues; the truncated
scanners scan a batch of <nreads> reads of 100-400 nt (cmgb_ScanBatch, pass 4:
5' and 3' truncation).  Runs the scan twice (the first builds the plan) and
prints the kernel time.  With tile_rows/arena the launch shape is fixed
(arena 1 shared, 2 global); without them the standard scanners let the
autotuner pick it and the truncated scanners use the default shape.
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
    q = 1 if algo in ("cyk", "trcyk") else 2
    m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", f"{name}.model.npz"))
    rng = np.random.default_rng(1)
    sc = lib.Scanner(0)
    shape = None
    if len(argv) > 5:
        cps = int(argv[6]) if len(argv) > 6 else 0
        sc.set_shape(int(argv[4]), 0, cps, 0, int(argv[5]))
        shape = (int(argv[4]), int(argv[5])) + ((cps,) if cps else ())
    if algo == "learned":
        # the default bench line's step on a <length>-residue target (both
        # strands): filter, CYK on the kept regions, Inside on survivors
        import torch
        from . import prefilter
        wts = prefilter.load(os.path.join(ROOT, "infernal_gb300", "filters", f"{name}.filter.npz"))
        f = prefilter.Prefilter(sc, wts, m.W)
        ins = [emit.sample(m, rng) for _ in range(max(1, L // 80000))]
        dsq, _ = emit.make_target(rng, L, (0.35, 0.60), ins)
        buf = prefilter.strand_buffer(dsq)
        d = torch.from_numpy(buf).cuda()
        torch.cuda.synchronize()
        if shape is None:
            sc.autotune(m, 1, "cyk"); sc.autotune(m, 2, "inside")
        for _ in range(2):
            t = time.time()
            hits, st = prefilter.filtered_scan(sc, f, m, d.data_ptr(), len(buf), prefilter.CYK_CUT, prefilter.INS_CUT)
            print(f"{name} L={L} learned kernel_ms={st['kernel_ms']} kept={st['kept']} cyk_residues={sum(st['lengths']['cyk'])} "
                  f"hits={sum(len(x) for x in hits)} wall_s={time.time() - t:.2f}")
        f.close()
    elif algo == "filter":
        import torch
        from . import prefilter
        wts = prefilter.load(os.path.join(ROOT, "infernal_gb300", "filters", f"{name}.filter.npz"))
        dsq, _ = emit.make_target(rng, L, 0.40, [])
        d = torch.from_numpy(dsq).cuda()
        f = prefilter.Prefilter(sc, wts, m.W)
        for _ in range(2):
            t = time.time()
            lg, ms = f.logits(d.data_ptr(), 1, L)
            print(f"{name} L={L} filter windows={len(lg)} kept={(lg > f.thr).mean():.4f} kernel_ms={ms:.2f} "
                  f"wall_s={time.time() - t:.2f}")
        f.close()
    elif algo.startswith("tr"):
        reads = [cmfile.digitize("".join(rng.choice(list("ACGU"), int(rng.integers(100, 401))))) for _ in range(L)]
        for _ in range(2):
            t = time.time()
            rs = sc.scan_batch(m, reads, algo=algo, qdbidx=q, pass_idx=4, cutoff=10.0)
            print(f"{name} reads={L} {algo} shape={shape} kernel_ms={rs[0].kernel_ms:.2f} wall_s={time.time() - t:.2f} "
                  f"hits={sum(len(r.hits) for r in rs)}")
    else:
        dsq, _ = emit.make_target(rng, L, 0.40, [])
        if shape is None:
            shape = sc.autotune(m, q, algo)
        for _ in range(2):
            t = time.time()
            r = sc.scan(m, dsq, 1, L, algo=algo, qdbidx=q, cutoff=10.0)
            print(f"{name} L={L} {algo} shape={shape} kernel_ms={r.kernel_ms:.2f} wall_s={time.time() - t:.2f} hits={len(r.hits)}")
    sc.close()


if __name__ == "__main__":
    main(sys.argv)
