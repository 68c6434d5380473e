"""cmsearch's search pipeline without HMM filters (cmsearch --nohmm) over the
GPU scanners.

Per target sequence and strand (src/cm_pipeline.c, cm_Pipeline :1600-1690):

1. CYK filter (pli_cyk_seq_filter, :3500-3600): FastCYKScan over the whole
   sequence at the QDB1 bands, NULL3 as configured, cutoff = the bit score
   whose P-value is F6 under the CYK calibration of the model's mode
   (mu_extrap + log(F6) / -lambda of ECMLC, or ECMGC for glocal models).
2. Survivor windows: each CYK hit (start i, stop j) becomes
   [max(1, j - (W-1)), min(L, i + (W-1))]; in position order, a window is
   merged with the next while the next one starts inside it.
3. Final stage (pli_final_stage, :3647): FastIInsideScan at the QDB2 bands on
   every window, cutoff T (0 bits, or the bit score of E when the search
   size Z is given, as cm_pli_NewModelThresholds does), all windows of a
   strand in one batched launch.
4. P-values and E-values from the Inside calibration of the model's mode
   (ECMLI / ECMGI): E = Z / dbsize * nrandhits * exp(-lambda (S - mu_extrap)),
   Z = residues searched (both strands unless top strand only); hits with
   E <= the threshold are reported in E-value order.

Truncated-hit passes are off in this mode, as in cmsearch --nohmm
(src/cm_pipeline.c:742-756).
"""
from __future__ import annotations

import math
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

import numpy as np

from . import emit, lib


@dataclass
class SearchHit:
    target: str
    strand: str            # "+" or "-"
    sfrom: int             # coordinates on the target's top strand (sfrom > sto on "-")
    sto: int
    score: float
    pvalue: float
    evalue: float
    root: int


def cyk_windows(hits: Sequence[tuple], W: int, L: int) -> List[Tuple[int, int]]:
    """Survivor windows of pli_cyk_seq_filter: hits (start, stop, ...) in
    position order (start, then stop: cm_tophits_SortByPosition for hits on
    the searched strand) padded by W-1 and merged while the next window
    starts at or before the current window's end (which becomes the merged
    hit's)."""
    hs = sorted(hits, key=lambda h: (h[0], h[1]))
    out, k = [], 0
    while k < len(hs):
        iwin = max(1, hs[k][1] - (W - 1))
        jwin = min(L, hs[k][0] + (W - 1))
        while k + 1 < len(hs) and max(1, hs[k + 1][1] - (W - 1)) <= jwin:
            k += 1
            jwin = min(L, hs[k][0] + (W - 1))
        out.append((iwin, jwin))
        k += 1
    return out


def _ecm(m, stage: str):
    local = bool(m.flags & 1)
    tag = {"cyk": "ECMLC" if local else "ECMGC", "inside": "ECMLI" if local else "ECMGI"}[stage]
    if tag not in m.ecm:
        raise ValueError(f"model {m.name} has no {tag} calibration (run calibrate first)")
    return m.ecm[tag]


def search(scanner: "lib.Scanner", m, targets: Sequence[Tuple[str, np.ndarray]], E: float = 10.0, F6: float = 1e-4,
           Z: Optional[float] = None, toponly: bool = False, null3: bool = True) -> List[SearchHit]:
    """Searches digital targets (name, Easel dsq with sentinels) with model m;
    returns the hits with E-value <= E, best first."""
    lc, li = _ecm(m, "cyk"), _ecm(m, "inside")
    cyk_cut = float(lc[1] + math.log(F6) / (-lc[0]))
    total = sum(len(d) - 2 for _, d in targets) * (1 if toponly else 2)
    z = float(Z) if Z is not None else float(total)
    T = lib.bits_at_evalue(li, E, z) if Z is not None else 0.0
    out: List[SearchHit] = []
    for name, dsq in targets:
        L = len(dsq) - 2
        strands = [("+", dsq)] if toponly else [("+", dsq), ("-", emit.revcomp_dsq(dsq))]
        for strand, d in strands:
            r = scanner.scan(m, d, 1, L, algo="cyk", qdbidx=1, cutoff=cyk_cut, do_null3=null3, env_cutoff=cyk_cut)
            wins = cyk_windows(r.hits, m.W, L)
            if not wins:
                continue
            pieces = [np.concatenate([[255], d[a:b + 1], [255]]).astype(np.uint8) for a, b in wins]
            rs = scanner.scan_batch(m, pieces, algo="inside", qdbidx=2, cutoff=T, do_null3=null3, env_cutoff=T)
            for (a, b), rw in zip(wins, rs):
                for h in rw.hits:
                    i, j = h[0] + a - 1, h[1] + a - 1
                    sfrom, sto = (i, j) if strand == "+" else (L - i + 1, L - j + 1)
                    p = math.exp(-li[0] * (h[4] - li[1]))
                    ev = lib.evalue(li, h[4], z)
                    if ev <= E:
                        out.append(SearchHit(name, strand, sfrom, sto, float(h[4]), min(1.0, p), ev, h[2]))
    out.sort(key=lambda x: (x.evalue, -x.score))
    return out


def scan_models(scanner: "lib.Scanner", models: Sequence, targets: Sequence[Tuple[str, np.ndarray]], E: float = 10.0,
                F6: float = 1e-4, toponly: bool = False, null3: bool = True) -> List[Tuple[int, SearchHit]]:
    """cmscan's --nohmm search: every model against every target, each target
    searched as its own database (Z = its residues on both strands, as cmscan
    computes E-values per query sequence).  The CYK filter of every (model,
    strand) pair runs in one multi-model launch (cmgb_ScanMulti); each
    model's final Inside runs on all of its windows in one batched launch.
    Returns (model index, hit) pairs, per target best E-value first; each
    (model, target) pair gives exactly search(scanner, model, [target]).
    """
    seqs, where = [], []                     # strands in launch order: (target index, strand, length)
    for t, (name, dsq) in enumerate(targets):
        L = len(dsq) - 2
        seqs.append(dsq); where.append((t, "+", L))
        if not toponly:
            seqs.append(emit.revcomp_dsq(dsq)); where.append((t, "-", L))
    cuts = []
    for m in models:
        lc = _ecm(m, "cyk")
        cuts.append(float(lc[1] + math.log(F6) / (-lc[0])))
    rs = scanner.scan_multi(list(models), seqs, algo="cyk", qdbidx=1, cutoffs=cuts, do_null3=null3,
                            env_cutoff=0.0)
    nseq = len(seqs)
    per_target: List[List[Tuple[int, SearchHit]]] = [[] for _ in targets]
    for a, m in enumerate(models):
        li = _ecm(m, "inside")
        wins = []                            # (strand index, a, b)
        for q in range(nseq):
            wins += [(q, a0, b0) for a0, b0 in cyk_windows(rs[a * nseq + q].hits, m.W, where[q][2])]
        if not wins:
            continue
        pieces = [np.concatenate([[255], seqs[q][a0:b0 + 1], [255]]).astype(np.uint8) for q, a0, b0 in wins]
        ri = scanner.scan_batch(m, pieces, algo="inside", qdbidx=2, cutoff=0.0, do_null3=null3, env_cutoff=0.0)
        for (q, a0, b0), rw in zip(wins, ri):
            t, strand, L = where[q]
            z = float(L * (1 if toponly else 2))
            for h in rw.hits:
                i, j = h[0] + a0 - 1, h[1] + a0 - 1
                sfrom, sto = (i, j) if strand == "+" else (L - i + 1, L - j + 1)
                ev = lib.evalue(li, h[4], z)
                if ev <= E:
                    p = math.exp(-li[0] * (h[4] - li[1]))
                    per_target[t].append((a, SearchHit(targets[t][0], strand, sfrom, sto, float(h[4]), min(1.0, p), ev, h[2])))
    out: List[Tuple[int, SearchHit]] = []
    for lst in per_target:
        out += sorted(lst, key=lambda x: (x[1].evalue, -x[1].score))
    return out
