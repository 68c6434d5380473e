"""Benchmark of the plain GPU QDB scan (CYK filter + Inside on survivors).

Workload (one "step"): a seeded synthetic target of --mb megabases at 40% GC
with CM-emitted sequences embedded on random strands, scanned on BOTH strands
with the clen-305 Plant_SRP CM (939 states, 4 bifurcations; the stand-in for
the synthetic clen-300 multibranch CM of the single-large-CM configuration):
  1. FastCYKScan, QDB1 bands (beta 1e-7), NULL3, greedy, filter cutoff
  2. survivor hits padded by W-1 and merged into windows
     (pli_cyk_seq_filter, src/cm_pipeline.c:3566-3601)
  3. FastIInsideScan, QDB2 bands (beta 1e-15), NULL3, greedy, on each window.
The default 10 steps x 2 Mb scan a 20 Mb slice of the configuration's 100 Mb
target distribution (the rate does not depend on the slice length once every
SM holds a window).

Metric: residues scanned per second (both strands counted) and GCUPS (DP
cells per second).  `value` uses residues already resident in device memory
(the *_dev entry points); `e2e` calls the host-buffer C ABI (host->device
copy of the residues and device->host hit lists inside every call).

`--workload trunc` runs the truncated-mode batch configuration instead: the
same CM against --reads reads per step of length uniform 100-400 nt (30%
CM-emitted sequences cut at a random 5' and/or 3' point, the rest iid ACGU at
50% GC), each read scanned by RefTrCYKScan (QDB1) for passes 2, 3 and 4
(5'-only, 3'-only, 5'+3' truncation) through the batched entry point
(cmgb_ScanBatch, one launch per pass), and reads with a CYK survivor rescanned
by RefITrInsideScan (QDB2) for that pass.  Residues count once per pass.

`--workload multi` runs the uneven multi-model batch: a panel of the
reference's calibrated CMs (clen 71-307; --cm-slots repeats them up to a
larger count) against --seqs sequences per step (log-uniform 100-5,000 nt,
45% GC, 5% carrying an emitted hit, both strands), every (CM, sequence) pair
by FastCYKScan QDB1 in one multi-model persistent launch (cmgb_ScanMulti),
timed beside one cmgb_ScanBatch launch per CM over the same sequences.
Residues count once per (CM, sequence) pair.

`--impl reference` times the reference's scanner on the host cores instead:
the reference's own FastCYKScan/FastIInsideScan compiled from source
(oracle/_ref) where that library exists, otherwise the C restatement of them
(oracle/cm_scan_oracle.c), one process per core, on a bounded sample of the
same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CYK_CUT = 10.0      # CYK filter threshold in bits (stand-in for the F6 E-value cutoff)
INS_CUT = 15.0      # final Inside threshold in bits


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


def rank_step_seed(rank, step):
    """Seed of one rank's step: every replica scans its own targets (weak
    scaling; no data is exchanged between ranks)."""
    return rank * 100000 + step


def max_over_ranks(values, world, device="cuda"):
    """Each entry's maximum over all ranks (the slowest replica's time); the
    only collective of a multi-GPU run, outside the timed region."""
    if world == 1:
        return [float(v) for v in values]
    import torch
    t = torch.tensor([float(v) for v in values], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(x) for x in t]


def make_step_input(model_glob, step, mb, seed=20261203, hits_per_mb=2.0, gc=0.40):
    """One step's target and its reverse complement: iid background at GC gc
    (or per-50-kb segments of GC drawn from a (low, high) range) with
    hits_per_mb emitted sequences embedded on random strands."""
    from infernal_gb300 import emit
    rng = np.random.default_rng([seed, step])
    L = int(mb * 1_000_000)
    nhits = max(1, int(round(hits_per_mb * mb)))     # default: 200 hits per 100 Mb
    ins = [emit.sample(model_glob, rng) for _ in range(nhits)]
    dsq, spans = emit.make_target(rng, L, gc, ins)
    return dsq, emit.revcomp_dsq(dsq)


def windows_from_hits(hits, W, L):
    """Survivor windows of the CYK filter: hits padded by W-1 and merged as
    pli_cyk_seq_filter does (src/cm_pipeline.c:3566-3601)."""
    from infernal_gb300 import pipeline
    return [list(w) for w in pipeline.cyk_windows(hits, W, L)]


def make_reads(model_glob, step, nreads, seed=20261204):
    """Reads of the truncated-mode batch: uniform 100-400 nt, 30% emitted
    sequences cut at a random 5' and/or 3' point, the rest iid at 50% GC."""
    from infernal_gb300 import cmfile, emit
    rng = np.random.default_rng([seed, step])
    out = []
    for k in range(nreads):
        n = int(rng.integers(100, 401))
        if rng.random() < 0.3:
            s = emit.sample(model_glob, rng)
            cut = int(rng.integers(0, 3))            # 0: 5' cut, 1: 3' cut, 2: both
            a = int(rng.integers(1, max(2, len(s) // 2))) if cut in (0, 2) else 0
            b = len(s) - int(rng.integers(1, max(2, len(s) // 2))) if cut in (1, 2) else len(s)
            frag = s[a:b] if b - a >= 20 else s
            if rng.random() < 0.5:
                frag = emit.revcomp(frag)
            pad = "".join(rng.choice(list("ACGU"), max(0, n - len(frag))))
            seq = (frag + pad)[:max(n, len(frag))] if cut == 1 else (pad + frag)[-max(n, len(frag)):]
        else:
            seq = "".join(rng.choice(list("ACGU"), n))
        out.append(cmfile.digitize(seq))
    return out


def run_trunc(args, rank, world):
    """Truncated-mode batch: TrCYK for passes 2/3/4 over every read, TrInside on survivors."""
    import torch
    from infernal_gb300 import cmfile, lib as L
    import ctypes
    m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", "Plant_SRP.model.npz"))
    torch.cuda.set_device(0 if world == 1 else _env_int("LOCAL_RANK", 0))
    sc = L.Scanner(torch.cuda.current_device())
    keep = []
    desc = cmfile.make_desc(m, keep=keep)
    nsteps = args.warmup + args.steps
    inputs = [make_reads(m, rank_step_seed(rank, s), args.reads) for s in range(nsteps)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    lib = sc.lib

    def cells_tr(q, n):   # truncated bands: d = 1 .. min(jp, dmax, W) for every non-E state
        dmax = m.dmax1 if q == 1 else m.dmax2
        dx = np.minimum(np.asarray(dmax, np.int64), m.W)[np.asarray(m.sttype) != cmfile.E_st]
        full = np.where(n <= dx, n * (n + 1) // 2, dx * (dx + 1) // 2 + (n - dx) * dx)
        return int(full.sum())

    cell_cache = {}

    def cells(q, n):
        if (q, n) not in cell_cache:
            cell_cache[(q, n)] = cells_tr(q, n)
        return cell_cache[(q, n)]

    def step(reads):
        kms, launches, cl, nh, res = 0.0, 0, 0, 0, 0
        for p in (2, 3, 4):
            rs = sc.scan_batch(m, reads, algo="trcyk", qdbidx=1, pass_idx=p, cutoff=CYK_CUT, env_cutoff=CYK_CUT)
            kms += rs[0].kernel_ms if rs else 0.0; launches += sc.last_launches()
            res += sum(len(d) - 2 for d in reads)
            cl += sum(cells(1, len(d) - 2) for d in reads)
            surv = [reads[q] for q, r in enumerate(rs) if r.hits]
            if surv:
                r2 = sc.scan_batch(m, surv, algo="trinside", qdbidx=2, pass_idx=p, cutoff=INS_CUT, env_cutoff=INS_CUT)
                kms += r2[0].kernel_ms; launches += sc.last_launches()
                cl += sum(cells(2, len(d) - 2) for d in surv)
                nh += sum(len(r.hits) for r in r2)
        return res, cl, kms, launches, nh

    for s in range(args.warmup):
        step(inputs[s])
    clk = start_clock_sampler(rank)
    tot, res, cl, kms, launches, nh = 0.0, 0, 0, 0.0, 0, 0
    for s in range(args.warmup, nsteps):
        flush.fill_(float(s))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r_, c_, k_, l_, h_ = step(inputs[s])
        torch.cuda.synchronize()
        tot += time.perf_counter() - t0
        res += r_; cl += c_; kms += k_; launches += l_; nh += h_
    clocks = stop_clock_sampler(clk)
    value = res / (kms / 1e3) / 1e6
    e2e = res / tot / 1e6
    out = {
        "metric": "Mres/s scanned (per pass), truncated-mode batch: RefTrCYKScan passes 2/3/4 + RefITrInsideScan on survivors",
        "value": round(value, 3), "unit": "Mres/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(kms / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (TrCYK) + int32 (TrInside)", "data": "synthetic",
        "config": {"workload": f"Plant_SRP CM stand-in (M={m.M}, clen={m.clen}, W={m.W}), {args.reads} reads/step "
                               f"uniform 100-400 nt, 30% emitted and cut 5'/3', rest iid GC 0.50; TrCYK QDB1 cutoff {CYK_CUT} "
                               f"-> TrInside QDB2 cutoff {INS_CUT}; passes 2,3,4; batched (cmgb_ScanBatch)",
                   "l2": "flushed between timed steps (256 MB write)", "parallelism": "1 GPU"},
        "gcups": round(cl / (kms / 1e3) / 1e9, 2),
        "e2e": {"value": round(e2e, 3), "unit": "Mres/s", "note": "wall time of the host-buffer batch calls"},
        "gpu_launches": launches, "hits_per_step": nh / args.steps, "clocks": clocks,
        "note": "value uses device kernel time (CUDA events); e2e includes host<->device copies and host hit resolution",
    }
    if rank == 0 and not args.no_cpu_baseline:
        import oracle
        use_ref = os.path.exists(oracle.REF_SO)
        reads = inputs[args.warmup]
        t0 = time.perf_counter()
        n = 0; k = 0
        while time.perf_counter() - t0 < args.cpu_seconds and k < len(reads):
            d = reads[k]
            oracle.tr_scan(m, d, 1, len(d) - 2, algo="trcyk", qdbidx=1, pass_idx=4, cutoff=CYK_CUT,
                           env_cutoff=CYK_CUT, reference=use_ref)
            n += len(d) - 2; k += 1
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(n / dt / 1e6, 6), "unit": "Mres/s", "cores": 1,
                               "kind": "reference" if use_ref else "port",
                               "sample": f"RefTrCYKScan QDB1 pass 4 over the first {k} reads of one step"}
    sc.close()
    return out


def _overlap(a, b):
    return max(0, min(a[1], b[1]) - max(a[0], b[0]) + 1)


def run_learned(args, rank, world):
    """Learned pre-filter + batched CYK -> Inside on the kept regions, against
    the plain scan of everything on the same targets (which measures the hit loss)."""
    import torch
    from infernal_gb300 import cmfile, lib as L, prefilter
    m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", "Plant_SRP.model.npz"))
    wts = prefilter.load(args.filter or os.path.join(ROOT, "infernal_gb300", "filters", "Plant_SRP.filter.npz"))
    torch.cuda.set_device(0)
    sc = L.Scanner(0)
    filt = prefilter.Prefilter(sc, wts, m.W)
    if args.filter_recall is not None:
        filt.use_recall(args.filter_recall)
    nsteps = args.warmup + args.steps
    inputs = [make_step_input(m, 500000 + s, args.mb, hits_per_mb=args.hits_per_mb, gc=(0.35, 0.60))
              for s in range(nsteps)]
    Lres = len(inputs[0][0]) - 2
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    sc.autotune(m, 1, "cyk"); sc.autotune(m, 2, "inside")

    def regions_scan(dsq, regs, algo, qdb, cut):
        """Batched scan of sub-ranges [a, b] of one strand; hits in strand coordinates."""
        if not regs:
            return [], 0.0
        buf = np.ascontiguousarray(dsq, np.uint8)
        offs = np.array([a - 1 for a, b in regs], np.int64)
        lens = np.array([b - a + 1 for a, b in regs], np.int64)
        import ctypes
        nh = np.zeros(len(regs), np.int64)
        hl = sc.lib.cmgb_hitlist_create()
        err = ctypes.create_string_buffer(256)
        st = sc.lib.cmgb_ScanBatch(sc._ctx, sc.model(m), err, L.BATCH_ALGOS[algo], qdb, 0, buf.ctypes.data, len(buf),
                                   offs.ctypes.data, lens.ctypes.data, len(regs), cut, hl, 1, cut, nh.ctypes.data,
                                   None, None, None, None)
        if st != 0:
            raise L.ScanError(st, err.value.decode())
        hits, h, k = [], L.Hit(), 0
        for q in range(len(regs)):
            for _ in range(int(nh[q])):
                sc.lib.cmgb_hitlist_get(hl, k, ctypes.byref(h)); k += 1
                hits.append((h.start + int(offs[q]), h.stop + int(offs[q]), h.score))
        sc.lib.cmgb_hitlist_destroy(hl)
        return hits, float(sc.lib.cmgb_ctx_last_kernel_ms(sc._ctx))

    def filtered_step(strands, dptrs):
        out, ms, kept = [], 0.0, 0
        for dsq, ptr in zip(strands, dptrs):
            logit, fms = filt.logits(ptr, 1, Lres)
            ms += fms
            regs = filt.regions(logit, 1, Lres)
            kept += sum(b - a + 1 for a, b in regs)
            cyk, k1 = regions_scan(dsq, regs, "cyk", 1, CYK_CUT)
            wins = windows_from_hits([(h[0], h[1]) for h in cyk], m.W, Lres)
            ins, k2 = regions_scan(dsq, wins, "inside", 2, INS_CUT)
            ms += k1 + k2
            out.append(ins)
        return out, ms, kept

    def plain_step(strands, dptrs):
        out = []
        for dsq, ptr in zip(strands, dptrs):
            r = sc.scan(m, dsq, 1, Lres, algo="cyk", qdbidx=1, cutoff=CYK_CUT, env_cutoff=CYK_CUT, device_ptr=ptr)
            ins = []
            for a, b in windows_from_hits(r.hits, m.W, Lres):
                r2 = sc.scan(m, dsq, a, b, algo="inside", qdbidx=2, cutoff=INS_CUT, env_cutoff=INS_CUT, device_ptr=ptr)
                ins += [(h[0], h[1], h[4]) for h in r2.hits]
            out.append(ins)
        return out

    dev = [[torch.from_numpy(x).to("cuda") for x in inp] for inp in inputs]
    torch.cuda.synchronize()
    for s in range(args.warmup):
        filtered_step(inputs[s], [t.data_ptr() for t in dev[s]])
    clk = start_clock_sampler(rank)
    tot, kms, kept, fhits = 0.0, 0.0, 0, []
    for s in range(args.warmup, nsteps):
        flush.fill_(float(s))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        h, k, kp = filtered_step(inputs[s], [t.data_ptr() for t in dev[s]])
        torch.cuda.synchronize()
        tot += time.perf_counter() - t0
        kms += k; kept += kp; fhits.append(h)
    clocks = stop_clock_sampler(clk)
    # the hit-loss reference: the plain scan of everything on the same steps (timed too)
    t0 = time.perf_counter()
    phits = [plain_step(inputs[s], [t.data_ptr() for t in dev[s]]) for s in range(args.warmup, nsteps)]
    t_plain = time.perf_counter() - t0
    # E <= 0.01 at this search size from the CM's local Inside calibration
    # (ECMLI line of Plant_SRP.c.cm: lambda, mu_extrap, calibration db size,
    # random hits): E = nrandhits * Z / dbsize * exp(-lambda (S - mu)), Z = residues per step
    lam, mu, cdb, nrand = 0.70748, -9.17856, 1600000.0, 519142.0
    e_bits = mu - np.log(0.01 / (nrand * (2 * Lres) / cdb)) / lam
    nplain = nfound = ne = nef = 0
    for ph, fh in zip(phits, fhits):
        for sp, sf in zip(ph, fh):
            for h in sp:
                found = any(_overlap(h, g) >= 0.5 * (h[1] - h[0] + 1) for g in sf)
                nplain += 1; nfound += found
                if h[2] >= e_bits:
                    ne += 1; nef += found
    res = 2 * Lres * args.steps
    value = res / tot / 1e6
    out = {
        "metric": "Mres/s scanned (both strands): learned pre-filter + batched QDB-CYK + Inside vs the plain GPU scan",
        "value": round(value, 3), "unit": "Mres/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * tot / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 (filter) + f32 (CYK) + int32 (Inside)", "data": "synthetic",
        "config": {"workload": f"Plant_SRP CM stand-in, {args.mb} Mb x 2 strands per step, GC varying 0.35-0.60 "
                               f"per 50 kb segment, "
                               f"{args.hits_per_mb} emitted hits per Mb; filter threshold "
                               f"{filt.thr:.3f} (validation recall {args.filter_recall or 0.99} of windows with an "
                               f"E <= 0.01 hit); kept regions scanned by CYK QDB1 ({CYK_CUT} bits) -> Inside QDB2 ({INS_CUT} bits)",
                   "l2": "flushed between timed steps (256 MB write)", "parallelism": "1 GPU"},
        "plain_mres_s": round(res / t_plain / 1e6, 3),
        "speedup_vs_plain": round(t_plain / tot, 2),
        "fraction_scanned": round(kept / res, 4),
        "hits_plain": nplain, "hits_found": nfound,
        "hit_loss": round(1.0 - nfound / nplain, 4) if nplain else None,
        "e001_bits": round(float(e_bits), 2), "e001_hits_plain": ne, "e001_hits_found": nef,
        "e001_hit_loss": round(1.0 - nef / ne, 4) if ne else None,
        "kernel_ms_per_step": round(kms / args.steps, 3),
        "clocks": clocks,
    }
    filt.close(); sc.close()
    return out


PANEL = ["tRNA", "Vault", "Plant_SRP", "tRNA1415G", "snR75", "tRNA-Sec", "srp-euk", "rnaseP-eubact",
         "5S_rRNA", "Cobalamin", "tRNA5", "tRNA5-hand"]


def load_panel():
    from infernal_gb300 import cmfile
    out = []
    for n in PANEL:
        p = os.path.join(ROOT, "tests", "golden", f"{n}.model.npz")
        if not os.path.exists(p):
            p = os.path.join(ROOT, "tests", "golden", "panel", f"{n}.model.npz")
        out.append(cmfile.load_npz(p))
    return out


def make_multi_seqs(models, step, nseq, seed=20261205):
    """Sequences of the uneven multi-model workload: lengths log-uniform
    100-5,000 nt, iid at 45% GC, 5% carrying an emitted hit of a random
    panel model; returned with their reverse complements (both strands)."""
    from infernal_gb300 import cmfile, emit
    rng = np.random.default_rng([seed, step])
    p = [0.275, 0.225, 0.225, 0.275]
    top = []
    for k in range(nseq):
        n = int(np.exp(rng.uniform(np.log(100), np.log(5000))))
        seq = "".join(rng.choice(list("ACGU"), n, p=p))
        if rng.random() < 0.05:
            h = emit.sample(models[int(rng.integers(len(models)))], rng)
            pos = int(rng.integers(0, max(1, n - len(h))))
            seq = (seq[:pos] + h + seq[pos + len(h):])[:max(n, len(h))]
        top.append(cmfile.digitize(seq))
    return top + [emit.revcomp_dsq(d) for d in top]


def run_multi(args, rank, world):
    """Uneven multi-model batch: every panel model x every sequence (both
    strands) by CYK QDB1 in one multi-model persistent launch per step,
    against one cmgb_ScanBatch launch per model over the same sequences."""
    import ctypes
    import torch
    from infernal_gb300 import cmfile, lib as L
    torch.cuda.set_device(0)
    sc = L.Scanner(0)
    models = load_panel()
    nslots = args.cm_slots or len(models)
    slots = [models[k % len(models)] for k in range(nslots)]
    nsteps = args.warmup + args.steps
    inputs = [make_multi_seqs(models, s, args.seqs) for s in range(nsteps)]
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    tuned = {n: sc.autotune(m, 1, "cyk") for n, m in zip(PANEL, models)}
    keep = []
    descs = [cmfile.make_desc(m, keep=keep) for m in models]
    cut = [CYK_CUT] * nslots

    def work(seqs):
        res = sum(len(d) - 2 for d in seqs) * nslots
        cells = 0
        for k in range(nslots):
            dk = descs[k % len(models)]
            cells += sum(sc.lib.cmgb_count_cells(ctypes.byref(dk), 1, len(d) - 2) for d in seqs)
        return res, cells

    for s in range(args.warmup):
        sc.scan_multi(slots, inputs[s], algo="cyk", qdbidx=1, cutoffs=cut, env_cutoff=CYK_CUT)
    clk = start_clock_sampler(rank)
    tot = kms = 0.0
    res = cells = launches = nh = 0
    h2d = d2h = 0
    for s in range(args.warmup, nsteps):
        flush.fill_(float(s))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rs = sc.scan_multi(slots, inputs[s], algo="cyk", qdbidx=1, cutoffs=cut, env_cutoff=CYK_CUT)
        tot += time.perf_counter() - t0
        kms += rs[0].kernel_ms
        launches += sc.last_launches()
        h2d, d2h = sc.last_transfer_bytes()
        nh += sum(len(r.hits) for r in rs)
        r_, c_ = work(inputs[s]); res += r_; cells += c_
    clocks = stop_clock_sampler(clk)
    # the same jobs as one batched launch per model
    t_per = kms_per = 0.0
    for s in range(args.warmup, nsteps):
        flush.fill_(float(s))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for m in slots:
            r = sc.scan_batch(m, inputs[s], algo="cyk", qdbidx=1, cutoff=CYK_CUT, env_cutoff=CYK_CUT)
            kms_per += r[0].kernel_ms
        t_per += time.perf_counter() - t0
    value = res / (kms / 1e3) / 1e6
    nlen = [len(d) - 2 for d in inputs[args.warmup]]
    out = {
        "metric": "Mres/s scanned (model x residue pairs, both strands), multi-model batched QDB-CYK in one persistent launch",
        "value": round(value, 3), "unit": "Mres/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(kms / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"{nslots} CM slots over a {len(models)}-CM panel of the reference's calibrated CMs "
                               f"(clen 71-307), {args.seqs} sequences x 2 strands per step, length log-uniform "
                               f"100-5000 (mean {np.mean(nlen):.0f}), GC 0.45, 5% with an emitted hit; "
                               f"CYK QDB1 cutoff {CYK_CUT} bits, NULL3, greedy; autotuned shapes per CM",
                   "model_residues_per_step": res // args.steps, "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": "1 GPU"},
        "gcups": round(cells / (kms / 1e3) / 1e9, 2),
        "e2e": {"value": round(res / tot / 1e6, 3), "unit": "Mres/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "per_model_batches": {"value": round(res / (kms_per / 1e3) / 1e6, 3), "unit": "Mres/s",
                              "wall_mres_s": round(res / t_per / 1e6, 3), "launches_per_step": nslots,
                              "note": "one cmgb_ScanBatch launch per CM over the same sequences"},
        "speedup_vs_per_model": round(kms_per / kms, 3) if kms > 0 else None,
        "gpu_launches": launches,
        "hits_per_step": nh / args.steps,
        "tuned_shapes": {k: {"tile_rows": v[0], "arena": "global" if v[1] == 2 else "shared"} for k, v in tuned.items()},
        "clocks": clocks,
    }
    sc.close()
    return out


# ----------------------------------------------------------------------------
def run_ours(args, rank, world):
    import torch
    from infernal_gb300 import cmfile, lib as L
    mpath = os.path.join(ROOT, "tests", "golden", "Plant_SRP.model.npz")
    m = cmfile.load_npz(mpath)
    torch.cuda.set_device(0 if world == 1 else _env_int("LOCAL_RANK", 0))
    dev = torch.cuda.current_device()
    sc = L.Scanner(dev)
    keep = []
    desc = cmfile.make_desc(m, keep=keep)
    lib = sc.lib
    import ctypes

    nsteps = args.warmup + args.steps
    inputs = [make_step_input(m, rank_step_seed(rank, s), args.mb) for s in range(nsteps)]
    Lres = len(inputs[0][0]) - 2
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # untimed set-up: the autotuner picks the tile shape of each band set / algorithm
    tuned = {"cyk_qdb1": sc.autotune(m, 1, "cyk"), "inside_qdb2": sc.autotune(m, 2, "inside")}
    xfer = [0, 0]

    opr = {1: dp_ops_per_residue(m, 1), 2: dp_ops_per_residue(m, 2)}
    ops_acc = [0]

    def step(strands, dev_ptrs):
        """One pass; returns (hits, cells, kernel_ms, launches)."""
        cells = 0
        kms = 0.0
        launches = 0
        nh = 0
        xfer[0] = xfer[1] = 0
        for k, dsq in enumerate(strands):
            ptr = dev_ptrs[k] if dev_ptrs else None
            r = sc.scan(m, dsq, 1, Lres, algo="cyk", qdbidx=1, cutoff=CYK_CUT, env_cutoff=CYK_CUT,
                        device_ptr=ptr)
            kms += r.kernel_ms; launches += sc.last_launches()
            hb, db = sc.last_transfer_bytes(); xfer[0] += hb; xfer[1] += db
            cells += lib.cmgb_count_cells(ctypes.byref(desc), 1, Lres)
            ops_acc[0] += opr[1] * Lres
            for a, b in windows_from_hits(r.hits, m.W, Lres):
                r2 = sc.scan(m, dsq, a, b, algo="inside", qdbidx=2, cutoff=INS_CUT, env_cutoff=INS_CUT,
                             device_ptr=ptr)
                kms += r2.kernel_ms; launches += sc.last_launches()
                hb, db = sc.last_transfer_bytes(); xfer[0] += hb; xfer[1] += db
                cells += lib.cmgb_count_cells(ctypes.byref(desc), 2, b - a + 1)
                ops_acc[0] += opr[2] * (b - a + 1)
                nh += len(r2.hits)
        return nh, cells, kms, launches

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def timed(use_dev):
        dev_inputs = []
        if use_dev:
            for s in range(nsteps):
                dev_inputs.append([torch.from_numpy(x).to("cuda") for x in inputs[s]])
        torch.cuda.synchronize()
        for s in range(args.warmup):
            step(inputs[s], [t.data_ptr() for t in dev_inputs[s]] if use_dev else None)
        tot, cells, kms, launches, nh = 0.0, 0, 0.0, 0, 0
        ops_acc[0] = 0
        for s in range(args.warmup, nsteps):
            flush.fill_(float(s))                  # evict L2 between timed steps
            barrier()
            t0 = time.perf_counter()
            h, c, k, l = step(inputs[s], [t.data_ptr() for t in dev_inputs[s]] if use_dev else None)
            barrier()
            tot += time.perf_counter() - t0
            cells += c; kms += k; launches += l; nh += h
        del dev_inputs
        return tot, cells, kms, launches, nh

    clk = start_clock_sampler(rank)
    t_dev, cells, kms, launches, nh = timed(True)
    ops = ops_acc[0]
    clocks = stop_clock_sampler(clk)
    t_e2e, _, _, _, _ = timed(False)
    h2d_step, d2h_step = xfer[0], xfer[1]     # transfers of the last host-buffer step
    t_dev, t_e2e = max_over_ranks([t_dev, t_e2e], world)
    res_per_rank = 2 * Lres * args.steps
    total_res = res_per_rank * world
    value = total_res / t_dev / 1e6
    e2e = total_res / t_e2e / 1e6
    out = {
        "metric": "Mres/s scanned (both strands), plain GPU QDB-CYK + Inside scan",
        "value": round(value, 3), "unit": "Mres/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * t_dev / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (CYK) + int32 (Inside)", "data": "synthetic",
        "config": {"workload": f"Plant_SRP CM stand-in (M={m.M}, clen={m.clen}, W={m.W}, 4 B), "
                               f"{args.mb} Mb x 2 strands per step, GC 0.40, {max(1, round(2 * args.mb))} emitted hits per step; "
                               f"CYK QDB1 cutoff {CYK_CUT} bits -> Inside QDB2 cutoff {INS_CUT} bits, NULL3, greedy",
                   "residues_per_step": 2 * Lres, "l2": "flushed between timed steps (256 MB write)",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"},
        "gcups": round(cells * world / t_dev / 1e9, 2),
        "kernel_gcups": round(cells / (kms / 1e3) / 1e9, 2) if kms > 0 else None,
        "kernel_ms_per_step": round(kms / args.steps, 3),
        "e2e": {"value": round(e2e, 3), "unit": "Mres/s", "h2d_bytes_per_step": h2d_step,
                "d2h_bytes_per_step": d2h_step},
        "tuned_shapes": {k: {"tile_rows": v[0], "arena": "global" if v[1] == 2 else "shared"} for k, v in tuned.items()},
        "gpu_launches": launches,
        "hits_per_step": nh / args.steps,
        "clocks": clocks,
    }
    out["roofline"] = roofline_block(cells, kms, Lres, args)
    out["alu_roofline"] = alu_roofline(ops, kms, clocks)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(m, inputs[args.warmup][0], threads=1, seconds=args.cpu_seconds)
    sc.close()
    return out


def work_per_d(m, qdbidx):
    """(cells[d], ops[d]) for d = 0..W: the DP cells of length d summed over
    the non-E states whose band holds d (QDB bands capped at W, MP from
    d = 2; src/cm_mx.c:5725-5738), and their algorithmic operations -- per
    non-B cell cnum adds + (cnum + 1) max/log-sum combines + 1 emission add
    if the state emits; per B cell one add and one combine per k term
    (k limits of src/cm_dpsearch.c:258-269, which depend on d only)."""
    from infernal_gb300 import cmfile
    W = m.W
    dmin, dmax = m.bands(qdbidx)
    cells = np.zeros(W + 1, np.int64)
    ops = np.zeros(W + 1, np.int64)
    d = np.arange(W + 1)
    for v in range(m.M):
        t = int(m.sttype[v])
        if t == cmfile.E_st:
            continue
        lo = 2 if t == cmfile.MP_st else 1
        if dmin is not None:
            lo = max(int(dmin[v]), lo)
        dn, dx = min(lo, W), (min(int(dmax[v]), W) if dmax is not None else W)
        if dx < dn:
            continue
        band = (d >= dn) & (d <= dx)
        cells += band
        if t == cmfile.B_st:
            w, y = int(m.cfirst[v]), int(m.cnum[v])
            if dmin is not None:
                kmin = np.maximum(0, np.maximum(min(int(dmin[y]), W), d - min(int(dmax[w]), W)))
                kmax = np.minimum(min(int(dmax[y]), W), d - min(int(dmin[w]), W))
            else:
                kmin, kmax = np.zeros_like(d), d
            ops += np.where(band, 2 * np.maximum(0, kmax - kmin + 1), 0)
        else:
            c = int(m.cnum[v])
            emits = t in (cmfile.MP_st, cmfile.ML_st, cmfile.MR_st, cmfile.IL_st, cmfile.IR_st)
            ops += band * (c + (c + 1) + (1 if emits else 0))
    return cells, ops


class Work:
    """Exact cells and operations of a scan of L residues with one band set:
    a cell (v, d) exists at every end position j >= d of the scanned range,
    so a scan of L residues holds sum_d max(0, L - d + 1) x per-d counts."""

    def __init__(self, m, qdbidx):
        self.c, self.o = work_per_d(m, qdbidx)
        d = np.arange(len(self.c), dtype=np.int64)
        # sum_{d<=n} (L + 1 - d) x[d] = (L + 1) S0(n) - S1(n)
        self.c0, self.c1 = np.cumsum(self.c), np.cumsum(self.c * d)
        self.o0, self.o1 = np.cumsum(self.o), np.cumsum(self.o * d)
        self.W = len(self.c) - 1

    def cells(self, L):
        n = min(int(L), self.W)
        return int((L + 1) * self.c0[n] - self.c1[n])

    def ops(self, L):
        n = min(int(L), self.W)
        return int((L + 1) * self.o0[n] - self.o1[n])


def dp_ops_per_residue(m, qdbidx):
    """Algorithmic DP operations per residue once j >= W."""
    return int(work_per_d(m, qdbidx)[1].sum())


def alu_roofline(ops, kms, clocks):
    """The DP's own roof: FP32/INT32 non-tensor issue (one operation per lane
    per clock; 152 SMs x 128 lanes)."""
    mhz = (clocks or {}).get("sm_max_mhz") or 2070.0
    peak = 152 * 128 * mhz * 1e6 / 1e12
    ach = ops / (kms / 1e3) / 1e12 if kms > 0 else 0.0
    return {"bound": "fp32/int32 non-tensor issue", "achieved": round(ach, 4), "peak": round(peak, 2),
            "unit": "Tops/s", "frac": round(ach / peak, 5),
            "note": "algorithmic DP operations (adds + max/log-sum combines) per kernel second"}


def roofline_block(cells, kms, Lres, args):
    """The scan kernel is not bandwidth bound: its algorithmic DRAM traffic is
    the residues (1 byte each) and the hit records; the DP state stays in
    shared memory / L2.  Reported against the measured HBM copy peak."""
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            peaks = json.load(fh)
    except OSError:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    alg_bytes = 2 * (Lres + 2) * args.steps
    ach = alg_bytes / (kms / 1e3) / 1e9 if kms > 0 else 0.0
    traffic = None
    prof = os.path.join(ROOT, "profiles", "qdb_scan_cyk_plant_srp_1mb_global.md")
    if os.path.exists(prof):      # DRAM bytes per residue of one ncu capture of the CYK kernel, scaled
        import re
        mt = re.search(r"^dram_bytes_per_residue:\s*([0-9.]+)", open(prof).read(), re.M)
        if mt:
            traffic = float(mt.group(1)) * (Lres + 2)     # per CYK launch (one strand)
    return {"bound": "hbm", "achieved": round(ach, 4), "peak": peak, "unit": "GB/s",
            "frac": round(ach / peak, 8), "traffic": traffic,
            "note": "algorithmic bytes = residues only; traffic = the CYK kernel's measured DRAM bytes per residue "
                    "(ncu, 1 Mb capture: tile-arena re-reads past L2) times the residues of one CYK launch; "
                    "the DP is bound by ALU issue and latency, see alu_roofline and the cell rate"}


def cpu_baseline(m, dsq, threads=1, seconds=10.0):
    """Times the CPU scanner (reference build if present, else the oracle port)
    on a prefix of one strand, sized to about `seconds` of work."""
    import oracle
    use_ref = os.path.exists(oracle.REF_SO)
    n = 2000
    t0 = time.perf_counter()
    oracle.scan(m, dsq, 1, n, algo="cyk", qdbidx=1, cutoff=CYK_CUT, env_cutoff=CYK_CUT, reference=use_ref)
    dt = time.perf_counter() - t0
    n2 = int(min(len(dsq) - 2, max(n, n * seconds / max(dt, 1e-3))))
    t0 = time.perf_counter()
    oracle.scan(m, dsq, 1, n2, algo="cyk", qdbidx=1, cutoff=CYK_CUT, env_cutoff=CYK_CUT, reference=use_ref)
    dt = time.perf_counter() - t0
    return {"value": round(n2 / dt / 1e6, 6), "unit": "Mres/s", "cores": threads,
            "kind": "reference" if use_ref else "port",
            "sample": f"FastCYKScan QDB1 over the first {n2} residues of one strand of the step-{0} target"}


def _ref_worker(argv):
    mb, idx, nres, use_ref = argv
    import oracle
    from infernal_gb300 import cmfile
    m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", "Plant_SRP.model.npz"))
    dsq, _ = make_step_input(m, 1000 + idx, min(mb, 0.1))
    t0 = time.perf_counter()
    oracle.scan(m, dsq, 1, nres, algo="cyk", qdbidx=1, cutoff=CYK_CUT, env_cutoff=CYK_CUT, reference=use_ref)
    return nres, time.perf_counter() - t0


def run_reference(args, rank, world):
    """CPU reference arm: all host cores, one process per core."""
    import multiprocessing as mp
    import oracle
    from infernal_gb300 import cmfile
    oracle.build_oracle()
    use_ref = os.path.exists(oracle.REF_SO)
    ncpu = len(os.sched_getaffinity(0))
    m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", "Plant_SRP.model.npz"))
    # size the per-process sample from a short single-process probe
    dsq, _ = make_step_input(m, 999, 0.01)
    t0 = time.perf_counter()
    oracle.scan(m, dsq, 1, 1500, algo="cyk", qdbidx=1, cutoff=CYK_CUT, reference=use_ref)
    rate = 1500 / (time.perf_counter() - t0)
    per_step_s = max(2.0, args.ref_step_seconds)
    nres = int(max(1500, min(90000, rate * per_step_s)))
    ctx = mp.get_context("spawn")
    times = []
    with ctx.Pool(ncpu) as pool:
        for s in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(_ref_worker, [(args.mb, s * ncpu + k, nres, use_ref) for k in range(ncpu)])
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                times.append((sum(r[0] for r in res), dt))
    tot_res = sum(t[0] for t in times)
    tot_t = sum(t[1] for t in times)
    v = tot_res / tot_t / 1e6
    return {
        "impl": "reference", "metric": "Mres/s scanned (both strands), plain GPU QDB-CYK + Inside scan",
        "value": round(v, 6), "unit": "Mres/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * tot_t / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (CYK)", "data": "synthetic",
        "config": {"workload": "same model and target distribution as the GPU arm; CYK QDB1 filter scan per core",
                   "parallelism": f"{ncpu} host processes"},
        "cpu_baseline": {"value": round(v, 6), "unit": "Mres/s", "cores": ncpu, "kind": "reference" if use_ref else "port",
                         "sample": f"{nres} residues per process per step, {ncpu} processes"},
        "e2e": {"value": round(v, 6), "unit": "Mres/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


_clk = {}


def start_clock_sampler(rank):
    if rank != 0:
        return None
    import tempfile
    fd, path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
    os.close(fd)
    try:
        fh = open(path, "w")
        p = subprocess.Popen(["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
                              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                              "--format=csv,noheader,nounits", "-lms", "200"], stdout=fh, stderr=subprocess.DEVNULL)
        return (p, fh, path)
    except Exception:
        os.unlink(path)
        return None


def stop_clock_sampler(h):
    if not h:
        return None
    p, fh, path = h
    p.terminate()
    p.wait()
    fh.close()
    sm, mx, reasons = [], 0, set()
    with open(path) as fh:
        lines = fh.readlines()
    os.unlink(path)
    for ln in lines:
        f = [x.strip() for x in ln.split(",")]
        if len(f) < 8:
            continue
        try:
            sm.append(float(f[1])); mx = max(mx, float(f[2]))
        except ValueError:
            continue
        for name, val in zip(("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"), f[4:8]):
            if val.lower().startswith("active"):
                reasons.add(name)
    if not sm:
        return None
    return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--mb", type=float, default=2.0, help="megabases of target per step (scanned on both strands)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-step-seconds", type=float, default=8.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="plain", choices=["plain", "trunc", "learned", "multi"],
                    help="plain: the single-large-CM scan (default); trunc: the truncated-mode read batch; "
                         "learned: the pre-filtered pipeline against the plain scan; multi: the uneven "
                         "multi-model batch")
    ap.add_argument("--seqs", type=int, default=300, help="sequences per step of the multi workload (x 2 strands)")
    ap.add_argument("--cm-slots", type=int, default=0, help="CM slots of the multi workload (default: the panel)")
    ap.add_argument("--reads", type=int, default=5000, help="reads per step of the trunc workload")
    ap.add_argument("--hits-per-mb", type=float, default=2.0, help="embedded hits per Mb (learned workload)")
    ap.add_argument("--filter", default=None, help="learned workload: filter weights (default: the shipped Plant_SRP filter)")
    ap.add_argument("--filter-recall", type=float, default=None,
                    help="learned workload: the filter's stored validation operating point to use "
                         "(recall of windows holding an E <= 0.01 hit; default: the file's threshold, 0.99)")
    args = ap.parse_args()
    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    if args.impl == "reference":
        if rank != 0:
            return
        print(json.dumps(run_reference(args, rank, world)))
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    if args.workload == "trunc":
        out = run_trunc(args, rank, world)
    elif args.workload == "learned":
        out = run_learned(args, rank, world)
    elif args.workload == "multi":
        out = run_multi(args, rank, world)
    else:
        out = run_ours(args, rank, world)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
