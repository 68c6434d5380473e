"""Benchmarks of the GPU QDB scanners; one JSON line per run.

Default workload (`--workload learned`, the learned-filter configuration):
each step is a seeded synthetic target of --mb megabases (GC drawn per 50 kb
segment from 0.35-0.60) with --hits-per-mb sequences emitted by the
clen-305 Plant_SRP CM (939 states, 4 bifurcations) embedded on random
strands, both strands held in device memory.  The learned pre-filter scores
every window of both strands, the kept regions of both strands get the QDB1
CYK scan (NULL3, greedy) in one batched launch, and the survivor windows of
the CYK hits (padded by W-1 and merged: pli_cyk_seq_filter,
src/cm_pipeline.c:3566-3601) get the QDB2 integer Inside scan in one more
launch.  The same targets then go through the plain GPU pipeline (the
single-launch CYK scan of each whole strand, then Inside on its survivor
windows), which judges what the filter loses: the hits with E <= 0.01 (the
model's Inside calibration, Z = all residues of the timed steps) that the
plain pipeline reports and the filtered one misses.

Other workloads: `plain` (the single-large-CM plain scan: Plant_SRP, GC
0.40, 2 hits per Mb), `cfg1` (Vault, the clen-100 stand-in, 1 Mb at GC 0.50
with 20 emitted hits, plain CYK -> Inside), `trunc` (the truncated-mode read
batch: passes 2/3/4 of RefTrCYKScan + RefITrInsideScan on survivors),
`multi` (the uneven multi-model batch in one persistent launch).

Metric: residues scanned per second (both strands counted) and GCUPS (DP
cells per second).  `value` uses residues already resident in device memory;
`e2e` copies each step's residues from pinned host memory inside the timed
region and reads every hit back to the host.

`--impl reference` times the reference's scanners on the host cores instead
(the reference's own FastCYKScan/FastIInsideScan compiled from source,
oracle/_ref, where that library exists, otherwise the C restatement of them,
oracle/cm_scan_oracle.c), one process per core, each step a bounded sample
of the same workload through the same CPU pipeline: CYK QDB1, then Inside
QDB2 on the survivor windows.
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


def make_step_input(model_glob, step, mb, seed=20261203, hits_per_mb=2.0, gc=0.40, nhits=None):
    """One step's target and its reverse complement: iid background at GC gc
    (or per-50-kb segments of GC drawn from a (low, high) range) with
    hits_per_mb emitted sequences (at least one; or exactly nhits) embedded
    on random strands."""
    from infernal_gb300 import emit
    rng = np.random.default_rng([seed, step])
    L = int(mb * 1_000_000)
    if nhits is None:
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


CYK_PROFILE = "qdb_scan_cyk_plant_srp_1mb_global.md"     # ncu summary giving the CYK kernel's DRAM bytes per residue

SPECS = {
    # model, target GC, default Mb per step, hits per Mb, learned filter?
    "learned": {"model": "Plant_SRP", "gc": (0.35, 0.60), "mb": 5.0, "hits_per_mb": 12.0, "filter": True, "seed": 500000},
    "plain": {"model": "Plant_SRP", "gc": 0.40, "mb": 2.0, "hits_per_mb": 2.0, "filter": False, "seed": 0},
    "cfg1": {"model": "Vault", "gc": 0.50, "mb": 1.0, "hits_per_mb": 20.0, "filter": False, "seed": 700000},
}


def spec_of(args):
    sp = dict(SPECS[args.workload])
    if args.mb is not None:
        sp["mb"] = args.mb
    if args.hits_per_mb is not None:
        sp["hits_per_mb"] = args.hits_per_mb
    sp["recall"] = args.filter_recall if args.filter_recall is not None else 0.99
    return sp


def load_model(name):
    from infernal_gb300 import cmfile
    p = os.path.join(ROOT, "tests", "golden", f"{name}.model.npz")
    if not os.path.exists(p):
        p = os.path.join(ROOT, "tests", "golden", "panel", f"{name}.model.npz")
    return cmfile.load_npz(p)


def pipeline_metric(sp):
    if sp["filter"]:
        return ("Mres/s scanned (both strands) on 1 GB300: learned pre-filter + batched QDB-CYK -> Inside, "
                "against the plain GPU scan at <= 1% loss of E <= 0.01 hits")
    return "Mres/s scanned (both strands) on 1 GB300: plain QDB-CYK -> Inside scan"


def pipeline_config(sp, m, world):
    gc = sp["gc"]
    gcs = f"GC varying {gc[0]}-{gc[1]} per 50 kb segment" if isinstance(gc, tuple) else f"GC {gc}"
    w = (f"{m.name} CM (M={m.M}, clen={m.clen}, W={m.W}), {sp['mb']} Mb x 2 strands per step, {gcs}, "
         f"{sp['hits_per_mb']} emitted hits per Mb embedded on random strands; ")
    if sp["filter"]:
        w += (f"learned BF16 window pre-filter at its validation operating point of recall {sp['recall']} "
              f"(windows holding a hit with E <= 0.01 at this search's size); kept regions of both strands -> ")
    w += f"QDB1 CYK ({CYK_CUT} bits, NULL3, greedy) -> survivor windows -> QDB2 integer Inside ({INS_CUT} bits)"
    return {"workload": w, "residues_per_step": int(2 * round(sp["mb"] * 1e6)),
            "l2": "flushed between timed steps (256 MB write)",
            "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except (OSError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def kernel_block(name, bound, achieved, peak, unit, note, traffic=None):
    return {"kernel": name, "bound": bound, "achieved": round(achieved, 4), "peak": round(peak, 3), "unit": unit,
            "frac": round(achieved / peak, 5) if peak else None, "traffic": traffic, "note": note}


def profile_dram_per_residue(name):
    """DRAM bytes per scanned residue of a kernel, from its committed ncu summary."""
    import re
    p = os.path.join(ROOT, "profiles", name)
    if not os.path.exists(p):
        return None
    mt = re.search(r"^dram_bytes_per_residue:\s*([0-9.]+)", open(p).read(), re.M)
    return float(mt.group(1)) if mt else None


def run_pipeline(args, rank, world):
    """learned / plain / cfg1: the CYK -> Inside pipeline over both strands of
    each step's target, with (learned) or without the pre-filter."""
    import torch
    from infernal_gb300 import lib as L, prefilter
    sp = spec_of(args)
    m = load_model(sp["model"])
    dev = 0 if world == 1 else _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(dev)
    sc = L.Scanner(dev)
    filt = None
    # E <= 0.01 at this search's size (every residue of the timed steps, both
    # strands) by the model's Inside calibration: the hits the filter must keep
    e_bits = float(L.bits_at_evalue(m.ecm["ECMLI"], 0.01, 2.0 * round(sp["mb"] * 1e6) * args.steps))
    if sp["filter"]:
        wts = prefilter.load(args.filter or os.path.join(ROOT, "infernal_gb300", "filters", f"{m.name}.filter.npz"))
        filt = prefilter.Prefilter(sc, wts, m.W)
        if filt.points is not None:
            filt.use_recall(sp["recall"], bits=e_bits)
    nsteps = args.warmup + args.steps
    inputs = [prefilter.strand_buffer(make_step_input(m, rank_step_seed(rank, sp["seed"] + s), sp["mb"],
                                                      hits_per_mb=sp["hits_per_mb"], gc=sp["gc"])[0])
              for s in range(nsteps)]
    nbuf = len(inputs[0])
    Lres = (nbuf - 3) // 2
    host = [torch.from_numpy(x).pin_memory() for x in inputs]
    devb = [h.to("cuda") for h in host]
    dstage = torch.empty(nbuf, dtype=torch.uint8, device="cuda")        # e2e: each step's copy lands here
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    tuned = {"cyk_qdb1": sc.autotune(m, 1, "cyk"), "inside_qdb2": sc.autotune(m, 2, "inside")}
    work = {"cyk": Work(m, 1), "inside": Work(m, 2)}

    def run(ptr):
        if filt is not None:
            return prefilter.filtered_scan(sc, filt, m, ptr, nbuf, CYK_CUT, INS_CUT)
        return prefilter.plain_scan(sc, m, ptr, nbuf, CYK_CUT, INS_CUT)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for s in range(args.warmup):
        run(devb[s].data_ptr())
    # timed: residues resident in device memory
    clk = start_clock_sampler(rank)
    tot, hits, sts = 0.0, [], []
    for s in range(args.warmup, nsteps):
        flush.fill_(float(s))
        barrier()
        t0 = time.perf_counter()
        h, st = run(devb[s].data_ptr())
        barrier()
        tot += time.perf_counter() - t0
        hits.append(h); sts.append(st)
    clocks = stop_clock_sampler(clk)
    # e2e: the step's residues copied from pinned host memory inside the timed region
    t_e2e, h2d, d2h = 0.0, 0, 0
    for s in range(args.warmup, nsteps):
        flush.fill_(float(s))
        barrier()
        t0 = time.perf_counter()
        dstage.copy_(host[s], non_blocking=True)
        torch.cuda.current_stream().synchronize()     # the scans run on the library's own stream
        h, st = run(dstage.data_ptr())
        barrier()
        t_e2e += time.perf_counter() - t0
        h2d += nbuf + st["h2d"]; d2h += st["d2h"]
    t_dev, t_e2e = max_over_ranks([tot, t_e2e], world)
    res = 2 * Lres * args.steps
    kms = {k: sum(st["kernel_ms"][k] for st in sts) for k in ("filter", "cyk", "inside")}
    lens = {k: [n for st in sts for n in st["lengths"][k]] for k in ("cyk", "inside")}
    ops = {k: sum(work[k].ops(n) for n in lens[k]) for k in lens}
    cells = {k: sum(work[k].cells(n) for n in lens[k]) for k in lens}
    launches = sum(st["launches"] for st in sts)
    out = {
        "metric": pipeline_metric(sp),
        "value": round(res * world / t_dev / 1e6, 3), "unit": "Mres/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * t_dev / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": ("bf16 (filter) + " if filt else "") + "f32 (CYK) + int32 (Inside)", "data": "synthetic",
        "config": pipeline_config(sp, m, world),
        "gcups": round((cells["cyk"] + cells["inside"]) * world / t_dev / 1e9, 2),
        "e2e": {"value": round(res * world / t_e2e / 1e6, 3), "unit": "Mres/s",
                "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps)},
        "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in kms.items()},
        "stage_wall_ms_per_step": {k: round(sum(st["wall_ms"][k] for st in sts) / args.steps, 3) for k in ("filter", "cyk", "inside")},
        "fraction_scanned": round(sum(st["kept"] for st in sts) / res, 4),
        "gpu_launches": launches,
        "tuned_shapes": {k: {"tile_rows": v[0], "arena": "global" if v[1] == 2 else "shared"} for k, v in tuned.items()},
        "clocks": clocks,
    }
    # roofline: measured issue peaks (this device) and the measured tensor peak
    peaks, pkind = measured_peaks()
    f32, i32 = sc.issue_peak("f32") / 1e12, sc.issue_peak("i32") / 1e12
    blocks = {}
    if kms["cyk"] > 0:
        ncall = max(1, sum(st["calls"]["cyk"] for st in sts))
        tr = profile_dram_per_residue(CYK_PROFILE)
        blocks["cyk"] = kernel_block("qdb_scan_kernel<CYK>", "fp32 add+max issue", ops["cyk"] / (kms["cyk"] / 1e3) / 1e12,
                                     f32, "Tops/s", "algorithmic DP operations of the CYK cells scanned, per kernel "
                                     "second (CUDA events); peak: cmgb_measure_issue_peak fp32 on this device; "
                                     "traffic: DRAM bytes per residue of the committed ncu summary x residues per launch",
                                     traffic=round(tr * sum(lens["cyk"]) / ncall) if tr else None)
    if kms["inside"] > 0:
        blocks["inside"] = kernel_block("qdb_scan_kernel<IInside>", "int32 add+max issue",
                                        ops["inside"] / (kms["inside"] / 1e3) / 1e12, i32, "Tops/s",
                                        "algorithmic operations (adds + ILogsum combines) per kernel second; "
                                        "peak: cmgb_measure_issue_peak int32 on this device")
    if filt is not None and kms["filter"] > 0:
        nwin = sum(-(-Lres // m.W) for _ in range(2)) * args.steps
        flops = 2.0 * nwin * (2 * m.W) * 9 * 128 * 128 * 5
        blocks["filter"] = kernel_block("filter_conv_tc (tcgen05)", "tensor", flops / (kms["filter"] / 1e3) / 1e12,
                                        float(peaks.get("bf16_tflops", 1900.0)), "TFLOP/s",
                                        f"dilated layers' GEMM FLOPs over the 2W positions of every window; peak: "
                                        f"{pkind} bf16 burst (MEASURED_PEAKS.json)")
    dom = max(blocks, key=lambda k: kms[k]) if blocks else None
    if dom:
        r = dict(blocks[dom])
        r["kernels"] = blocks
        r["dominant_share_of_kernel_time"] = round(kms[dom] / max(1e-9, sum(kms.values())), 3)
        r["peaks_measured"] = {"fp32_add_max_tops": round(f32, 2), "int32_add_max_tops": round(i32, 2),
                               "sm_count": torch.cuda.get_device_properties(dev).multi_processor_count}
        out["roofline"] = r
    if filt is not None:
        # the judge: the plain pipeline on the same targets
        run_plain = lambda ptr: prefilter.plain_scan(sc, m, ptr, nbuf, CYK_CUT, INS_CUT)
        run_plain(devb[0].data_ptr())
        t_plain, phits, pk = 0.0, [], 0.0
        for s in range(args.warmup, nsteps):
            flush.fill_(float(s))
            barrier()
            t0 = time.perf_counter()
            h, st = run_plain(devb[s].data_ptr())
            barrier()
            t_plain += time.perf_counter() - t0
            phits.append(h); pk += st["kernel_ms"]["cyk"] + st["kernel_ms"]["inside"]
        nplain = nfound = ne = nef = 0
        for ph, fh in zip(phits, hits):
            for sp_, sf in zip(ph, fh):
                for hh in sp_:
                    found = any(_overlap(hh, g) >= 0.5 * (hh[1] - hh[0] + 1) for g in sf)
                    nplain += 1; nfound += found
                    if hh[2] >= e_bits:
                        ne += 1; nef += found
        out.update({
            "plain_mres_s": round(res / t_plain / 1e6, 3),
            "speedup_vs_plain": round(t_plain / tot, 3),
            "plain_kernel_ms_per_step": round(pk / args.steps, 3),
            "e001_bits": round(e_bits, 2), "e001_hits_plain": ne, "e001_hits_found": nef,
            "e001_hit_loss": round(1.0 - nef / ne, 4) if ne else None,
            "hits_plain": nplain, "hits_found": nfound,
            "filter_threshold": round(filt.thr, 4),
        })
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(m, inputs[args.warmup][: Lres + 2], seconds=args.cpu_seconds)
    if filt is not None:
        filt.close()
    sc.close()
    return out


def _overlap(a, b):
    return max(0, min(a[1], b[1]) - max(a[0], b[0]) + 1)


MULTI_SPEC = {"models": ["Vault", "tRNA", "5S_rRNA", "Plant_SRP"], "gc": (0.35, 0.60), "mb": 2.0, "hits_per_mb": 30.0,
              "seed": 800000}


def multi_config(sp, models, world, recall):
    names = ", ".join(f"{m.name} (clen {m.clen}, W {m.W})" for m in models)
    return {"workload": f"{len(models)} CMs [{names}] against {sp['mb']} Mb x 2 strands per step, GC varying "
                        f"{sp['gc'][0]}-{sp['gc'][1]} per 50 kb segment, {sp['hits_per_mb']} emitted hits per Mb (the "
                        f"models in turn) on random strands; one BF16 filter trunk with a read-out per CM at its validation "
                        f"operating point of recall {recall}; every model's kept regions of both strands -> QDB1 CYK "
                        f"({CYK_CUT} bits) in one multi-model launch -> survivor windows -> QDB2 Inside ({INS_CUT} bits) in one "
                        f"multi-model launch",
            "residues_per_step": int(2 * round(sp["mb"] * 1e6)), "l2": "flushed between timed steps (256 MB write)",
            "parallelism": f"replicas x{world}" if world > 1 else "1 GPU"}


def make_step_input_multi(models, step, mb, seed, hits_per_mb, gc):
    """One step's target with hits emitted by the models in turn."""
    from infernal_gb300 import emit
    rng = np.random.default_rng([seed, step])
    L = int(mb * 1_000_000)
    nhits = max(len(models), int(round(hits_per_mb * mb)))
    ins = [emit.sample(models[k % len(models)], rng) for k in range(nhits)]
    dsq, spans = emit.make_target(rng, L, gc, ins)
    return dsq


def run_pipeline_multi(args, rank, world):
    """learned-multi: several CMs, one filter trunk with a head per CM, against
    the plain multi-model scan of the same targets."""
    import torch
    from infernal_gb300 import lib as L, prefilter
    sp = dict(MULTI_SPEC)
    if args.mb is not None:
        sp["mb"] = args.mb
    if args.hits_per_mb is not None:
        sp["hits_per_mb"] = args.hits_per_mb
    recall = args.filter_recall if args.filter_recall is not None else 0.99
    models = [load_model(n) for n in sp["models"]]
    K = len(models)
    dev = 0 if world == 1 else _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(dev)
    sc = L.Scanner(dev)
    wts = prefilter.load(args.filter or os.path.join(ROOT, "infernal_gb300", "filters", "multi4.filter.npz"))
    Wf = int(wts["W"])
    filt = prefilter.Prefilter(sc, wts, Wf)
    Z = 2.0 * round(sp["mb"] * 1e6) * args.steps
    e_bits = [float(L.bits_at_evalue(m.ecm["ECMLI"], 0.01, Z)) for m in models]
    pts = wts["recall_points"]                         # [K][rows][5]
    thr = []
    for k in range(K):
        p = pts[k]
        levels = np.unique(p[:, 0])
        lv = levels[levels <= e_bits[k]].max() if (levels <= e_bits[k]).any() else levels.min()
        row = p[(p[:, 0] == lv) & (np.abs(p[:, 1] - recall) < 1e-9)]
        thr.append(float(row[0, 2]))
    filt.thr = np.array(thr)
    nsteps = args.warmup + args.steps
    inputs = [prefilter.strand_buffer(make_step_input_multi(models, rank_step_seed(rank, sp["seed"] + s), sp["mb"], sp["seed"],
                                                            sp["hits_per_mb"], sp["gc"])) for s in range(nsteps)]
    nbuf = len(inputs[0])
    Lres = (nbuf - 3) // 2
    host = [torch.from_numpy(x).pin_memory() for x in inputs]
    devb = [h.to("cuda") for h in host]
    dstage = torch.empty(nbuf, dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    for m in models:
        sc.autotune(m, 1, "cyk"); sc.autotune(m, 2, "inside")
    work = {(k, a): Work(m, 1 if a == "cyk" else 2) for k, m in enumerate(models) for a in ("cyk", "inside")}
    run = lambda ptr: prefilter.filtered_scan_multi(sc, filt, models, ptr, nbuf)
    run_plain = lambda ptr: prefilter.plain_scan_multi(sc, models, ptr, nbuf)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for s in range(args.warmup):
        run(devb[s].data_ptr())
    clk = start_clock_sampler(rank)
    tot, hits, sts = 0.0, [], []
    for s in range(args.warmup, nsteps):
        flush.fill_(float(s)); barrier()
        t0 = time.perf_counter()
        h, st = run(devb[s].data_ptr())
        barrier()
        tot += time.perf_counter() - t0
        hits.append(h); sts.append(st)
    clocks = stop_clock_sampler(clk)
    t_e2e, h2d, d2h = 0.0, 0, 0
    for s in range(args.warmup, nsteps):
        flush.fill_(float(s)); barrier()
        t0 = time.perf_counter()
        dstage.copy_(host[s], non_blocking=True)
        torch.cuda.current_stream().synchronize()
        h, st = run(dstage.data_ptr())
        barrier()
        t_e2e += time.perf_counter() - t0
        h2d += nbuf + st["h2d"]; d2h += st["d2h"]
    run_plain(devb[0].data_ptr())
    t_plain, phits, pk = 0.0, [], 0.0
    for s in range(args.warmup, nsteps):
        flush.fill_(float(s)); barrier()
        t0 = time.perf_counter()
        h, st = run_plain(devb[s].data_ptr())
        barrier()
        t_plain += time.perf_counter() - t0
        phits.append(h); pk += st["kernel_ms"]["cyk"] + st["kernel_ms"]["inside"]
    t_dev, t_e2e, t_plain = max_over_ranks([tot, t_e2e, t_plain], world)
    res = 2 * Lres * args.steps
    kms = {a: sum(st["kernel_ms"][a] for st in sts) for a in ("filter", "cyk", "inside")}
    cells = sum(work[(k, a)].cells(n) for st in sts for a in ("cyk", "inside") for k, n in st["lengths"][a])
    ops = {a: sum(work[(k, a)].ops(n) for st in sts for k, n in st["lengths"][a]) for a in ("cyk", "inside")}
    per = {}
    for k, m in enumerate(models):
        ne = nef = 0
        for ph, fh in zip(phits, hits):
            for s_ in (0, 1):
                for hh in ph[k][s_]:
                    if hh[2] >= e_bits[k]:
                        ne += 1
                        nef += any(_overlap(hh, g) >= 0.5 * (hh[1] - hh[0] + 1) for g in fh[k][s_])
        per[m.name] = {"e001_bits": round(e_bits[k], 2), "hits_plain": ne, "hits_found": nef, "threshold": round(thr[k], 4)}
    ne = sum(v["hits_plain"] for v in per.values()); nef = sum(v["hits_found"] for v in per.values())
    peaks, pkind = measured_peaks()
    f32, i32 = sc.issue_peak("f32") / 1e12, sc.issue_peak("i32") / 1e12
    blocks = {}
    if kms["cyk"] > 0:
        blocks["cyk"] = kernel_block("qdb_scan_kernel<CYK, multi-model>", "fp32 add+max issue", ops["cyk"] / (kms["cyk"] / 1e3) / 1e12,
                                     f32, "Tops/s", "algorithmic DP operations of every model's CYK cells scanned, per kernel "
                                     "second; peak: cmgb_measure_issue_peak fp32 on this device")
    if kms["inside"] > 0:
        blocks["inside"] = kernel_block("qdb_scan_kernel<IInside, multi-model>", "int32 add+max issue",
                                        ops["inside"] / (kms["inside"] / 1e3) / 1e12, i32, "Tops/s",
                                        "algorithmic operations per kernel second; peak: cmgb_measure_issue_peak int32")
    if kms["filter"] > 0:
        nwin = 2 * (-(-Lres // Wf)) * args.steps
        flops = 2.0 * nwin * (2 * Wf) * 9 * 128 * 128 * 5
        blocks["filter"] = kernel_block("filter_conv_tc (tcgen05)", "tensor", flops / (kms["filter"] / 1e3) / 1e12,
                                        float(peaks.get("bf16_tflops", 1900.0)), "TFLOP/s",
                                        f"dilated layers' GEMM FLOPs over the 2W positions of every window; peak: {pkind} bf16 burst")
    out = {
        "metric": ("Mres/s scanned (both strands) on 1 GB300: learned pre-filter (one trunk, a head per CM) + batched "
                   "multi-model QDB-CYK -> Inside, against the plain multi-model GPU scan at <= 1% loss of E <= 0.01 hits"),
        "value": round(res * world / t_dev / 1e6, 3), "unit": "Mres/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * t_dev / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "bf16 (filter) + f32 (CYK) + int32 (Inside)", "data": "synthetic",
        "config": multi_config(sp, models, world, recall),
        "gcups": round(cells * world / t_dev / 1e9, 2),
        "e2e": {"value": round(res * world / t_e2e / 1e6, 3), "unit": "Mres/s",
                "h2d_bytes_per_step": int(h2d / args.steps), "d2h_bytes_per_step": int(d2h / args.steps)},
        "kernel_ms_per_step": {k: round(v / args.steps, 3) for k, v in kms.items()},
        "fraction_scanned": round(sum(st["kept"] for st in sts) / (res * K), 4),
        "gpu_launches": sum(st["launches"] for st in sts),
        "plain_mres_s": round(res / t_plain / 1e6, 3), "speedup_vs_plain": round(t_plain / tot, 3),
        "plain_kernel_ms_per_step": round(pk / args.steps, 3),
        "e001_hits_plain": ne, "e001_hits_found": nef, "e001_hit_loss": round(1.0 - nef / ne, 4) if ne else None,
        "per_model": per, "clocks": clocks,
    }
    if blocks:
        dom = max(blocks, key=lambda k: kms[k])
        r = dict(blocks[dom]); r["kernels"] = blocks
        r["dominant_share_of_kernel_time"] = round(kms[dom] / max(1e-9, sum(kms.values())), 3)
        r["peaks_measured"] = {"fp32_add_max_tops": round(f32, 2), "int32_add_max_tops": round(i32, 2),
                               "sm_count": torch.cuda.get_device_properties(dev).multi_processor_count}
        out["roofline"] = r
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
    # warm-up steps (plans, autotuned shapes, first-touch allocations) run on
    # at most 100 sequences: they are untimed and need every model, not volume
    inputs = [make_multi_seqs(models, s, args.seqs if s >= args.warmup else min(args.seqs, 100)) for s in range(nsteps)]
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
    for s in (range(args.warmup, nsteps) if not args.no_per_model else ()):
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
        "per_model_batches": None if args.no_per_model else {
            "value": round(res / (kms_per / 1e3) / 1e6, 3), "unit": "Mres/s",
            "wall_mres_s": round(res / t_per / 1e6, 3), "launches_per_step": nslots,
            "note": "one cmgb_ScanBatch launch per CM over the same sequences"},
        "speedup_vs_per_model": round(kms_per / kms, 3) if kms > 0 and not args.no_per_model else None,
        "gpu_launches": launches,
        "hits_per_step": nh / args.steps,
        "tuned_shapes": {k: {"tile_rows": v[0], "arena": "global" if v[1] == 2 else "shared"} for k, v in tuned.items()},
        "clocks": clocks,
    }
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


def cpu_pipeline(m, dsq, n, use_ref):
    """The CPU pipeline on residues 1..n of one strand: FastCYKScan QDB1
    (NULL3, greedy, cutoff CYK_CUT), then FastIInsideScan QDB2 on each
    survivor window (cutoff INS_CUT) -- the reference's scanners when
    use_ref, else their C restatement."""
    import oracle
    hits = oracle.scan(m, dsq, 1, n, algo="cyk", qdbidx=1, cutoff=CYK_CUT, env_cutoff=CYK_CUT, reference=use_ref)[0]
    nwin = 0
    for a, b in windows_from_hits(hits, m.W, n):
        oracle.scan(m, dsq, a, b, algo="inside", qdbidx=2, cutoff=INS_CUT, env_cutoff=INS_CUT, reference=use_ref)
        nwin += 1
    return nwin


def cpu_baseline(m, dsq, seconds=10.0):
    """The CPU pipeline (reference build if present, else the C restatement)
    on one host core over a prefix of one strand, sized to about `seconds`."""
    import oracle
    oracle.build_oracle()
    use_ref = os.path.exists(oracle.REF_SO)
    n = 2000
    t0 = time.perf_counter()
    cpu_pipeline(m, dsq, n, use_ref)
    dt = time.perf_counter() - t0
    n2 = int(min(len(dsq) - 2, max(n, n * seconds / max(dt, 1e-3))))
    t0 = time.perf_counter()
    nw = cpu_pipeline(m, dsq, n2, use_ref)
    dt = time.perf_counter() - t0
    return {"value": round(n2 / dt / 1e6, 6), "unit": "Mres/s", "cores": 1,
            "kind": "reference" if use_ref else "port",
            "sample": f"CYK QDB1 over the first {n2} residues of the first timed step's top strand, then Inside QDB2 "
                      f"on its {nw} survivor windows, one core"}


def _ref_worker_multi(argv):
    names, mb, hits_per_mb, gc, seed, nres, use_ref = argv
    models = [load_model(n) for n in names]
    nh = int(np.random.default_rng([seed, 1]).poisson(hits_per_mb * nres / 1e6))
    from infernal_gb300 import emit
    rng = np.random.default_rng([seed, 2])
    ins = [emit.sample(models[k % len(models)], rng) for k in range(nh)]
    dsq, _ = emit.make_target(rng, nres + 1000, gc, ins)
    t0 = time.perf_counter()
    for m in models:
        cpu_pipeline(m, dsq, nres, use_ref)
    return nres, time.perf_counter() - t0


def _ref_worker(argv):
    workload, mb, hits_per_mb, gc, seed, nres, use_ref = argv
    sp = SPECS[workload]
    m = load_model(sp["model"])
    mb = max(nres / 1e6, 0.002) + 0.001
    nh = int(np.random.default_rng([seed, 1]).poisson(hits_per_mb * nres / 1e6))   # the workload's hit density
    dsq, _ = make_step_input(m, seed, mb, hits_per_mb=hits_per_mb, gc=gc, nhits=nh)
    t0 = time.perf_counter()
    cpu_pipeline(m, dsq, nres, use_ref)
    return nres, time.perf_counter() - t0


def run_reference(args, rank, world):
    """CPU reference arm: the workload's CPU pipeline on all host cores, one
    process per core, each step a bounded sample of the workload."""
    import multiprocessing as mp
    import oracle
    if args.workload not in SPECS and args.workload != "learned-multi":
        return {"impl": "reference", "unavailable": f"the {args.workload} workload has no CPU reference arm here"}
    oracle.build_oracle()
    use_ref = os.path.exists(oracle.REF_SO)
    ncpu = len(os.sched_getaffinity(0))
    if args.workload == "learned-multi":
        return run_reference_multi(args, world, use_ref, ncpu)
    sp = spec_of(args)
    m = load_model(sp["model"])
    # size the per-process sample from a short single-process probe
    dsq, _ = make_step_input(m, 999, 0.01, hits_per_mb=0.0, gc=sp["gc"])
    t0 = time.perf_counter()
    cpu_pipeline(m, dsq, 1500, use_ref)
    rate = 1500 / (time.perf_counter() - t0)
    nres = int(max(1500, min(200000, rate * max(2.0, args.ref_step_seconds))))
    ctx = mp.get_context("spawn")
    times = []
    with ctx.Pool(ncpu) as pool:
        for s in range(args.warmup + args.steps):
            jobs = [(args.workload, sp["mb"], sp["hits_per_mb"], sp["gc"], 900000 + s * ncpu + k, nres, use_ref)
                    for k in range(ncpu)]
            t0 = time.perf_counter()
            res = pool.map(_ref_worker, jobs)
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                times.append((sum(r[0] for r in res), dt))
    tot_res = sum(t[0] for t in times)
    tot_t = sum(t[1] for t in times)
    v = tot_res / tot_t / 1e6
    return {
        "impl": "reference", "metric": pipeline_metric(sp),
        "value": round(v, 6), "unit": "Mres/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * tot_t / args.steps, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 (CYK) + int32 (Inside)", "data": "synthetic",
        "config": pipeline_config(sp, m, 1),
        "cpu_baseline": {"value": round(v, 6), "unit": "Mres/s", "cores": ncpu, "kind": "reference" if use_ref else "port",
                         "sample": f"per step {ncpu} processes, each: CYK QDB1 over {nres} residues of a fresh target of "
                                   f"this workload's distribution, then Inside QDB2 on its survivor windows "
                                   f"(the reference has no learned filter: its pipeline scans everything)"},
        "e2e": {"value": round(v, 6), "unit": "Mres/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference_multi(args, world, use_ref, ncpu):
    """CPU reference arm of learned-multi: every model's CYK -> Inside pipeline
    over the same bounded sample, one process per core (no filter: the
    reference scans everything with every model)."""
    import multiprocessing as mp
    sp = dict(MULTI_SPEC)
    if args.mb is not None:
        sp["mb"] = args.mb
    if args.hits_per_mb is not None:
        sp["hits_per_mb"] = args.hits_per_mb
    recall = args.filter_recall if args.filter_recall is not None else 0.99
    models = [load_model(n) for n in sp["models"]]
    t0 = time.perf_counter()
    _ref_worker_multi((sp["models"], sp["mb"], 0.0, sp["gc"], 998, 1000, use_ref))
    rate = 1000 / (time.perf_counter() - t0)
    nres = int(max(1000, min(100000, rate * max(2.0, args.ref_step_seconds))))
    times = []
    with mp.get_context("spawn").Pool(ncpu) as pool:
        for s in range(args.warmup + args.steps):
            jobs = [(sp["models"], sp["mb"], sp["hits_per_mb"], sp["gc"], 950000 + s * ncpu + k, nres, use_ref) for k in range(ncpu)]
            t0 = time.perf_counter()
            res = pool.map(_ref_worker_multi, jobs)
            dt = time.perf_counter() - t0
            if s >= args.warmup:
                times.append((sum(r[0] for r in res), dt))
    v = sum(t[0] for t in times) / sum(t[1] for t in times) / 1e6
    return {
        "impl": "reference", "metric": ("Mres/s scanned (both strands) on 1 GB300: learned pre-filter (one trunk, a head per "
                                        "CM) + batched multi-model QDB-CYK -> Inside, against the plain multi-model GPU scan "
                                        "at <= 1% loss of E <= 0.01 hits"),
        "value": round(v, 6), "unit": "Mres/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1000 * sum(t[1] for t in times) / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (CYK) + int32 (Inside)", "data": "synthetic",
        "config": multi_config(sp, models, 1, recall),
        "cpu_baseline": {"value": round(v, 6), "unit": "Mres/s", "cores": ncpu, "kind": "reference" if use_ref else "port",
                         "sample": f"per step {ncpu} processes, each: every model's CYK QDB1 over {nres} residues of a fresh "
                                   f"target of this workload's distribution, then Inside QDB2 on its survivor windows"},
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
    ap.add_argument("--mb", type=float, default=None, help="megabases of target per step, scanned on both strands "
                                                           "(default: the workload's)")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-step-seconds", type=float, default=8.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--workload", default="learned", choices=["learned", "learned-multi", "plain", "cfg1", "trunc", "multi"],
                    help="learned: the pre-filtered pipeline against the plain scan (default); plain: the "
                         "single-large-CM plain scan; cfg1: the clen-100 plain scan; trunc: the truncated-mode read "
                         "batch; multi: the uneven multi-model batch")
    ap.add_argument("--seqs", type=int, default=300, help="sequences per step of the multi workload (x 2 strands)")
    ap.add_argument("--cm-slots", type=int, default=0, help="CM slots of the multi workload (default: the panel)")
    ap.add_argument("--no-per-model", action="store_true", help="multi workload: skip the one-launch-per-CM comparison")
    ap.add_argument("--reads", type=int, default=5000, help="reads per step of the trunc workload")
    ap.add_argument("--hits-per-mb", type=float, default=None, help="embedded hits per Mb (default: the workload's)")
    ap.add_argument("--filter", default=None, help="learned workload: filter weights (default: the shipped filter)")
    ap.add_argument("--filter-recall", type=float, default=None,
                    help="learned workload: the filter's stored validation operating point to use "
                         "(recall of windows holding an E <= 0.01 hit; default 0.99)")
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
    elif args.workload == "multi":
        out = run_multi(args, rank, world)
    elif args.workload == "learned-multi":
        out = run_pipeline_multi(args, rank, world)
    else:
        out = run_pipeline(args, rank, world)
    if rank == 0:
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
