"""Learned window pre-filter ahead of the QDB-CYK stage.

The network (scored on the GPU by the hand-written kernels of
``csrc/filter.cu`` through ``cmgb_filter_windows``): windows of 2W residues at
stride W, one-hot ACGU, six dilated convolutions (kernel 9, dilations
1..32, 4 -> 128 -> 128 channels, ReLU), max over positions, linear read-out.
Weights and activations are BF16 with FP32 accumulation.

Training data come from the plain scanner itself: windows are labelled
positive when the plain QDB-CYK scan (cutoff ``CYK_CUT``) followed by the
QDB2 Inside scan (cutoff ``INS_CUT``) reports a hit in them.  Positives are windows holding sequences emitted by the CM (whole or
cut at random points) in background of varying GC; negatives are iid
background and dinucleotide-shuffled positives (the Altschul-Erickson
doublet-preserving shuffle, restated here).  Either PyTorch fits the
weights (``train``, with batch normalisation folded at export) or the
hand-written device trainer does (``train_native``, cmgb_filter_trainer_*,
no batch normalisation); only the exported arrays are used at scan time.

``filtered_scan`` is the pipeline: filter all windows of both strands, keep
those above the threshold, merge them into regions and run the plain
CYK -> Inside scan on the regions only.  The plain scan on everything
(``plain_scan``) stays the measure of what the filter misses.

    python -m infernal_gb300.prefilter train <model> <out.npz> [n_windows] [steps]
    python -m infernal_gb300.prefilter train-native <model> <out.npz> [n_windows] [steps]
    python -m infernal_gb300.prefilter train-bulk <model> <out.npz> [n_windows] [epochs]
    python -m infernal_gb300.prefilter train-bulk-multi <model,model,...> <out.npz> [n_windows] [epochs]
"""
from __future__ import annotations

import ctypes
import os
import sys
import time
from typing import List, Optional, Tuple

import numpy as np

from . import cmfile, emit, lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CYK_CUT = 10.0
INS_CUT = 15.0
E_BITS = 17.2     # Inside bits with E <= 0.01 in 4 Mb for Plant_SRP (ECMLI calibration of its CM file)
CH, KT, DIL = 128, 9, (1, 2, 4, 8, 16, 32)


# ---------------------------------------------------------------------------
# sequences
def dinuc_shuffle(seq: str, rng: np.random.Generator) -> str:
    """Doublet-preserving shuffle (Altschul & Erickson 1985): a random Euler
    path through the multigraph of the sequence's dinucleotides that starts
    and ends where the sequence does.  Last exit edges of every vertex but
    the final one form a random tree towards the final vertex; the other
    edges leave each vertex in random order."""
    if len(seq) < 3:
        return seq
    edges = {}
    for a, b in zip(seq[:-1], seq[1:]):
        edges.setdefault(a, []).append(b)
    last = seq[-1]
    verts = list(edges.keys())
    # random last-exit tree: for each vertex, pick a random exit such that
    # following last exits reaches `last` (Wilson-style loop-erased walks)
    in_tree = {last: True}
    last_exit = {}
    for v in verts:
        u = v
        path = {}
        while u not in in_tree:
            nxt = edges[u][int(rng.integers(len(edges[u])))]
            path[u] = nxt
            u = nxt
        u = v
        while u not in in_tree:
            last_exit[u] = path[u]
            in_tree[u] = True
            u = path[u]
    order = {}
    for v, outs in edges.items():
        outs = list(outs)
        if v in last_exit:
            outs.remove(last_exit[v])
            rng.shuffle(outs)
            outs.append(last_exit[v])
        else:
            rng.shuffle(outs)
        order[v] = outs[::-1]          # pop from the end
    out = [seq[0]]
    u = seq[0]
    while order.get(u):
        u = order[u].pop()
        out.append(u)
    return "".join(out)


def background(rng: np.random.Generator, n: int, gc: float) -> str:
    p = [(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2]
    return "".join(rng.choice(list("ACGU"), n, p=p))


def make_windows(m: cmfile.CMModel, n: int, rng: np.random.Generator, first: int = 0) -> List[np.ndarray]:
    """n training windows of 2W residues (window k of the set is kind
    (first + k) % 3): an emitted sequence (whole or cut at random 5'/3'
    points) at a random offset, iid background, or a dinucleotide-shuffled
    emitted-sequence window; GC drawn from 0.35-0.60 per window.  Every
    window gets a freshly emitted sequence, so no sequence repeats."""
    W2 = 2 * m.W
    out = []
    for k in range(first, first + n):
        gc = float(rng.uniform(0.35, 0.60))
        kind = k % 3
        if kind == 1:
            s = background(rng, W2, gc)
        else:
            e = emit.sample(m, rng)
            if rng.random() < 0.15 and len(e) > 40:
                a, b = sorted(int(x) for x in rng.integers(0, len(e) + 1, 2))
                e = e[a:b] if b - a >= 20 else e
            if rng.random() < 0.5:
                e = emit.revcomp(e)
            e = e[:W2]
            bg = background(rng, W2, gc)
            pos = int(rng.integers(0, W2 - len(e) + 1))
            s = bg[:pos] + e + bg[pos + len(e):]
            if kind == 2:
                s = dinuc_shuffle(s, rng)
        out.append(cmfile.digitize(s[:W2]))
    return out


def make_window_block(m: cmfile.CMModel, n: int, seed: int, first: int = 0) -> np.ndarray:
    """n training windows of 2W residues as rows of a uint8 array [n][2W + 2]
    (an Easel sentinel at both ends of each row), window k of kind
    (first + k) % 3 as in make_windows -- an emitted sequence (whole, or cut
    at random 5'/3' points 15% of the time; either strand) at a random offset
    in background, iid background, or the dinucleotide shuffle of such a
    window -- with the GC content of each window drawn from 0.35-0.60.
    Backgrounds are drawn in bulk and sequences come from emit.Sampler, so a
    million windows take minutes on a few cores."""
    import random
    rng = np.random.default_rng(seed)
    rnd = random.Random(seed)
    S = emit.Sampler(m)
    W2 = 2 * m.W
    gc = rng.uniform(0.35, 0.60, n)
    u = rng.random((n, W2))
    pa, pc = ((1 - gc) / 2)[:, None], (gc / 2)[:, None]
    codes = ((u >= pa).astype(np.uint8) + (u >= pa + pc) + (u >= pa + 2 * pc)).astype(np.uint8)
    out = np.full((n, W2 + 2), cmfile.DSQ_SENTINEL, np.uint8)
    out[:, 1:-1] = codes
    tr = bytes.maketrans(b"ACGU", b"\x00\x01\x02\x03")
    for k in range(n):
        kind = (first + k) % 3
        if kind == 1:
            continue
        e = S.sample(rnd)
        if rnd.random() < 0.15 and len(e) > 40:
            a, b = sorted((rnd.randrange(len(e) + 1), rnd.randrange(len(e) + 1)))
            e = e[a:b] if b - a >= 20 else e
        if rnd.random() < 0.5:
            e = emit.revcomp(e)
        e = e[:W2]
        pos = rnd.randrange(W2 - len(e) + 1)
        out[k, 1 + pos:1 + pos + len(e)] = np.frombuffer(e.encode().translate(tr), np.uint8)
        if kind == 2:
            s = "".join("ACGU"[x] for x in out[k, 1:-1])
            out[k, 1:-1] = np.frombuffer(dinuc_shuffle(s, rng).encode().translate(tr), np.uint8)
    return out


def _block_job(args):
    name, n, seed, first = args
    m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", f"{name}.model.npz"))
    return make_window_block(m, n, seed, first)


def make_window_block_parallel(name: str, n: int, seed: int, procs: int = 0) -> np.ndarray:
    """make_window_block over worker processes (spawned: call before any GPU use)."""
    import multiprocessing as mp
    procs = procs or max(1, min(16, os.cpu_count() or 1))
    per = -(-n // procs)
    per += (3 - per % 3) % 3                      # keep the kind cycle aligned across parts
    jobs = [(name, min(per, n - k * per), seed * 1000 + k, k * per) for k in range(procs) if k * per < n]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        parts = pool.map(_block_job, jobs)
    return np.concatenate(parts)


def best_inside_scores(sc: "lib.Scanner", m: cmfile.CMModel, block: np.ndarray, rows=None, chunk: int = 20000) -> np.ndarray:
    """Best final-stage score per window of a window block: the plain
    pipeline (QDB1 CYK at CYK_CUT, then QDB2 Inside at INS_CUT on the windows
    with a CYK hit, NULL3, greedy), batched; -inf where it reports no hit.
    rows: the windows to scan (default all); the others stay -inf."""
    n, width = block.shape
    best = np.full(n, -np.inf, np.float32)
    rows = np.arange(n) if rows is None else np.asarray(rows)
    for a in range(0, len(rows), chunk):
        r = rows[a:a + chunk]
        buf = np.concatenate([block[r].ravel(), np.full(1, cmfile.DSQ_SENTINEL, np.uint8)])
        offs = np.arange(len(r), dtype=np.int64) * width
        lens = np.full(len(r), width - 2, np.int64)
        rs = sc.scan_batch(m, None, algo="cyk", qdbidx=1, cutoff=CYK_CUT, env_cutoff=CYK_CUT, ranges=(buf, offs, lens))
        surv = np.array([q for q, x in enumerate(rs) if x.hits], np.int64)
        if len(surv):
            r2 = sc.scan_batch(m, None, algo="inside", qdbidx=2, cutoff=INS_CUT, env_cutoff=INS_CUT,
                               ranges=(buf, offs[surv], lens[surv]))
            for q, x in zip(surv, r2):
                if x.hits:
                    best[r[q]] = max(h[4] for h in x.hits)
    return best


def block_logits(f: "Prefilter", block: np.ndarray) -> np.ndarray:
    """The inference kernels' logits of every window of a block (windows
    placed back to back: a scan's even-numbered windows are the block's
    rows, each zero-padded at its ends as in training); [n] or [n][H]."""
    import torch
    n, width = block.shape
    out = np.empty((n, f.H), np.float32)
    step = 10000
    for a in range(0, n, step):
        body = block[a:a + step, 1:-1].ravel()
        seq = np.concatenate([[cmfile.DSQ_SENTINEL], body, [cmfile.DSQ_SENTINEL]]).astype(np.uint8)
        d = torch.from_numpy(seq).cuda()
        torch.cuda.synchronize()
        lg, _ = f.logits(d.data_ptr(), 1, len(seq) - 2)
        lg = lg.reshape(-1, f.H)
        out[a:a + step] = lg[0::2][: min(step, n - a)]
    return out[:, 0] if f.H == 1 else out


def operating_points(logit: np.ndarray, best: np.ndarray, background: np.ndarray,
                     bits=(15.0, 17.2, 20.0, 21.8, 25.0), recalls=(0.9, 0.95, 0.98, 0.99, 0.995, 0.999)) -> np.ndarray:
    """Rows (bits, recall, threshold, negatives kept, background kept): for
    windows whose best final-stage score is >= bits, the logit threshold
    that keeps the given fraction of them; negatives = windows with no
    final-stage hit, background = pure iid windows."""
    rows = []
    neg = ~np.isfinite(best)
    for b in bits:
        pos = np.sort(logit[best >= b])
        if len(pos) == 0:
            continue
        for q in recalls:
            t = float(pos[int((1 - q) * len(pos))] - 1e-3)
            rows.append((b, q, t, float((logit[neg] > t).mean()), float((logit[background] > t).mean())))
    return np.array(rows, np.float64)


# ---------------------------------------------------------------------------
# one filter for several CMs: a shared trunk and one read-out head per CM
def make_window_block_multi(models, n: int, seed: int, first: int = 0):
    """n windows of 2 Wmax residues (Wmax: the largest W of the models) for a
    several-head filter; window k is of kind (first + k) % (K + 2): kinds
    0..K-1 hold a sequence emitted by model k (whole, or cut 15% of the time;
    either strand) in background, kind K is iid background, kind K + 1 the
    dinucleotide shuffle of a window of a random model's kind.  GC 0.35-0.60
    per window.  Returns (block [n][2 Wmax + 2] with sentinels, source model
    per window: -1 for background, -2 for shuffled)."""
    import random
    K = len(models)
    rng = np.random.default_rng(seed)
    rnd = random.Random(seed)
    samplers = [emit.Sampler(m) for m in models]
    W2 = 2 * max(m.W for m in models)
    gc = rng.uniform(0.35, 0.60, n)
    u = rng.random((n, W2))
    pa, pc = ((1 - gc) / 2)[:, None], (gc / 2)[:, None]
    out = np.full((n, W2 + 2), cmfile.DSQ_SENTINEL, np.uint8)
    out[:, 1:-1] = ((u >= pa).astype(np.uint8) + (u >= pa + pc) + (u >= pa + 2 * pc)).astype(np.uint8)
    src = np.full(n, -1, np.int32)
    tr = bytes.maketrans(b"ACGU", b"\x00\x01\x02\x03")
    for k in range(n):
        kind = (first + k) % (K + 2)
        if kind == K:
            continue
        a = kind if kind < K else rnd.randrange(K)
        e = samplers[a].sample(rnd)
        if rnd.random() < 0.15 and len(e) > 40:
            x, y = sorted((rnd.randrange(len(e) + 1), rnd.randrange(len(e) + 1)))
            e = e[x:y] if y - x >= 20 else e
        if rnd.random() < 0.5:
            e = emit.revcomp(e)
        e = e[:W2]
        pos = rnd.randrange(W2 - len(e) + 1)
        out[k, 1 + pos:1 + pos + len(e)] = np.frombuffer(e.encode().translate(tr), np.uint8)
        src[k] = a
        if kind == K + 1:
            body = "".join("ACGU"[x] for x in out[k, 1:-1])
            out[k, 1:-1] = np.frombuffer(dinuc_shuffle(body, rng).encode().translate(tr), np.uint8)
            src[k] = -2
    return out, src


def _block_multi_job(args):
    names, n, seed, first = args
    models = [_load_model(x) for x in names]
    return make_window_block_multi(models, n, seed, first)


def _load_model(name: str) -> cmfile.CMModel:
    p = os.path.join(ROOT, "tests", "golden", f"{name}.model.npz")
    if not os.path.exists(p):
        p = os.path.join(ROOT, "tests", "golden", "panel", f"{name}.model.npz")
    return cmfile.load_npz(p)


def make_window_block_multi_parallel(names, n: int, seed: int, procs: int = 0):
    """make_window_block_multi over spawned worker processes."""
    import multiprocessing as mp
    procs = procs or max(1, min(16, os.cpu_count() or 1))
    cyc = len(names) + 2
    per = -(-n // procs)
    per += (cyc - per % cyc) % cyc
    jobs = [(list(names), min(per, n - k * per), seed * 1000 + k, k * per) for k in range(procs) if k * per < n]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        parts = pool.map(_block_multi_job, jobs)
    return np.concatenate([p[0] for p in parts]), np.concatenate([p[1] for p in parts])


def best_inside_scores_multi(sc: "lib.Scanner", models, block: np.ndarray, rows=None, chunk: int = 10000) -> np.ndarray:
    """[n][K] best final-stage score of every window under every model: the
    plain pipeline per model (QDB1 CYK at CYK_CUT on every (model, window)
    pair in one multi-model launch, then QDB2 Inside at INS_CUT on the pairs
    with a CYK hit); -inf where a model reports no hit."""
    n, width = block.shape
    K = len(models)
    best = np.full((n, K), -np.inf, np.float32)
    rows = np.arange(n) if rows is None else np.asarray(rows)
    for a in range(0, len(rows), chunk):
        r = rows[a:a + chunk]
        buf = np.concatenate([block[r].ravel(), np.full(1, cmfile.DSQ_SENTINEL, np.uint8)])
        offs = np.arange(len(r), dtype=np.int64) * width
        lens = np.full(len(r), width - 2, np.int64)
        jobs = [(k, q) for k in range(K) for q in range(len(r))]
        rs = sc.scan_multi(models, None, jobs=jobs, algo="cyk", qdbidx=1, cutoffs=[CYK_CUT] * K, env_cutoff=CYK_CUT,
                           ranges=(buf, offs, lens))
        surv = [(k, q) for (k, q), x in zip(jobs, rs) if x.hits]
        if surv:
            r2 = sc.scan_multi(models, None, jobs=surv, algo="inside", qdbidx=2, cutoffs=[INS_CUT] * K,
                               env_cutoff=INS_CUT, ranges=(buf, offs, lens))
            for (k, q), x in zip(surv, r2):
                if x.hits:
                    best[r[q], k] = max(h[4] for h in x.hits)
    return best


def train_bulk_multi(names, out: str, nwin: int, epochs: float, nval: int = 40000, seed: int = 20261207,
                     batch: int = 256, lr: float = 1e-3) -> None:
    """The several-head recipe: windows of every model's kind plus background
    and shuffles (make_window_block_multi), labelled per model by the plain
    pipeline (a final hit of at least INS_CUT bits under that model), one
    head per model trained together on the device, operating points per head
    from fresh validation windows scored by the inference kernels."""
    t0 = time.time()
    models = [_load_model(x) for x in names]
    K = len(models)
    Wf = max(m.W for m in models)
    block, src = make_window_block_multi_parallel(names, nwin, seed)       # before the first GPU call
    vblock, vsrc = make_window_block_multi_parallel(names, nval, seed + 1)
    print(f"{nwin} + {nval} windows of {2 * Wf} made in {time.time() - t0:.0f}s", flush=True)
    sc = lib.Scanner(0)
    for m in models:
        sc.autotune(m, 1, "cyk"); sc.autotune(m, 2, "inside")
    best = best_inside_scores_multi(sc, models, block, rows=np.nonzero(src != -1)[0])   # iid windows: no hit assumed
    vbest = best_inside_scores_multi(sc, models, vblock)
    y = (best >= INS_CUT).astype(np.float32)
    print(f"labelled in {time.time() - t0:.0f}s; positives per head {y.sum(0).astype(int).tolist()}; validation "
          f"{(vbest >= INS_CUT).sum(0).tolist()}", flush=True)
    posw = np.maximum(1.0, (y == 0).sum(0) / np.maximum(1.0, (y == 1).sum(0))).astype(np.float32)
    steps = int(epochs * nwin / batch)
    rng = np.random.default_rng(seed)
    tr = NativeTrainer(sc, Wf, batch, seed=seed + 1, heads=K)
    X = block[:, 1:-1]
    try:
        for it in range(steps):
            idx = rng.integers(0, nwin, batch)
            warm = max(1, steps // 10)
            f = (it + 1) / warm if it < warm else 0.5 * (1 + np.cos(np.pi * (it - warm) / max(1, steps - warm)))
            loss, ms = tr.step(X[idx], y[idx], posw, lr * f)
            if it % 500 == 0:
                print(f"step {it} loss {loss:.4f} ({ms:.1f} ms)", flush=True)
        wts = tr.weights()
    finally:
        tr.close()
    print(f"trained {steps} steps in {time.time() - t0:.0f}s", flush=True)
    f = Prefilter(sc, wts, Wf)
    vl = block_logits(f, vblock)
    f.close()
    pts = np.stack([operating_points(vl[:, k], vbest[:, k], vsrc == -1) for k in range(K)])
    for k in range(K):
        for r in pts[k]:
            if r[1] in (0.98, 0.99):
                print(f"  {names[k]}: bits {r[0]:5.1f} recall {r[1]:.3f}: threshold {r[2]:8.3f}, negatives kept "
                      f"{r[3]:.4f}, background kept {r[4]:.4f}", flush=True)
    thr = np.array([float(pts[k][(pts[k][:, 0] == 17.2) & (pts[k][:, 1] == 0.99)][0, 2]) for k in range(K)])
    save(wts, out, threshold=thr, W=Wf, models=np.array(list(names)), trained_windows=nwin, recall_points=pts,
         trainer=np.array("cmgb_filter_trainer (device, no batch normalisation, one head per model)"),
         recipe=np.array(f"prefilter.train_bulk_multi({list(names)!r}, nwin={nwin}, epochs={epochs}, nval={nval}, "
                         f"seed={seed}, batch={batch}, lr={lr})"))
    sc.close()
    print(f"saved {out} after {time.time() - t0:.0f}s", flush=True)


def label_windows(sc: "lib.Scanner", m: cmfile.CMModel, wins: List[np.ndarray], chunk: int = 2000) -> np.ndarray:
    """1 where the plain pipeline reports a final hit in the window: a
    QDB-CYK survivor (>= CYK_CUT) that the QDB2 Inside scan keeps (>= INS_CUT),
    i.e. the hits the filter must not lose."""
    lab = np.zeros(len(wins), np.float32)
    best = np.full(len(wins), -1e30, np.float32)
    for a in range(0, len(wins), chunk):
        rs = sc.scan_batch(m, wins[a:a + chunk], algo="cyk", qdbidx=1, cutoff=CYK_CUT, env_cutoff=CYK_CUT,
                           do_null3=True)
        surv = [a + q for q, r in enumerate(rs) if r.hits]
        if surv:
            r2 = sc.scan_batch(m, [wins[k] for k in surv], algo="inside", qdbidx=2, cutoff=INS_CUT,
                               env_cutoff=INS_CUT, do_null3=True)
            for k, r in zip(surv, r2):
                lab[k] = 1.0 if r.hits else 0.0
                if r.hits:
                    best[k] = max(h[4] for h in r.hits)
    label_windows.best = best
    return lab


def onehot(wins: List[np.ndarray]):
    import torch
    X = np.zeros((len(wins), 4, len(wins[0]) - 2), np.float32)
    for k, d in enumerate(wins):
        body = d[1:-1]
        ok = body < 4
        X[k, body[ok], np.nonzero(ok)[0]] = 1.0
    return torch.from_numpy(X)


# ---------------------------------------------------------------------------
# network (training only)
def make_net():
    import torch
    import torch.nn as nn

    class FilterNet(nn.Module):
        """Convolution -> batch norm -> ReLU per layer; the batch norms are
        folded into the convolutions' weights and biases at export."""
        def __init__(self):
            super().__init__()
            self.convs = nn.ModuleList()
            self.norms = nn.ModuleList()
            cin = 4
            for d in DIL:
                self.convs.append(nn.Conv1d(cin, CH, KT, dilation=d, padding=4 * d))
                self.norms.append(nn.BatchNorm1d(CH))
                cin = CH
            self.out = nn.Linear(CH, 1)

        def forward(self, x):
            for c, n in zip(self.convs, self.norms):
                x = torch.relu(n(c(x)))
            return self.out(x.amax(dim=2)).squeeze(1)
    return FilterNet()


def _folded(net, l):
    """Layer l's convolution with its (eval-mode) batch norm folded in:
    weight [co, ci, 9] and bias [co], float32."""
    c, n = net.convs[l], net.norms[l]
    scale = (n.weight / (n.running_var + n.eps).sqrt()).detach().float()
    w = c.weight.detach().float() * scale[:, None, None]
    b = (c.bias.detach().float() - n.running_mean.float()) * scale + n.bias.detach().float()
    return w.cpu(), b.cpu()


def export(net) -> dict:
    """Weights in the kernel layout (csrc/filter.cu)."""
    import torch
    net = net.eval()
    w0, b0 = _folded(net, 0)
    w0k = np.ascontiguousarray(w0.numpy().transpose(2, 1, 0))  # [9][4][128]
    ws, bs = [], [b0.numpy()]
    for l in range(1, 6):
        w, b = _folded(net, l)                                # [co, ci, 9]
        w = w.permute(2, 0, 1).contiguous().to(torch.bfloat16)  # [9][co][ci]
        ws.append(w.view(torch.int16).numpy().view(np.uint16))
        bs.append(b.numpy())
    wb = np.ascontiguousarray(np.stack(ws))                    # [5][9][128][128]
    bias = np.stack(bs).astype(np.float32)
    wout = np.concatenate([net.out.weight.detach().float().cpu().numpy().ravel(),
                           net.out.bias.detach().float().cpu().numpy().ravel()]).astype(np.float32)
    return {"w0": w0k.astype(np.float32), "w": wb, "bias": bias, "wout": wout}


def reference_logits(weights: dict, wins: List[np.ndarray]) -> np.ndarray:
    """The network in PyTorch FP32 on the exported weights, with the kernel's
    BF16 rounding points (weights of layers 2-6, every layer's output)."""
    import torch
    import torch.nn.functional as F
    dev = "cuda" if torch.cuda.is_available() else "cpu"
    x = onehot(wins).to(dev)
    w0 = torch.from_numpy(weights["w0"]).to(dev).permute(2, 1, 0).contiguous()   # [128, 4, 9]
    b = torch.from_numpy(weights["bias"]).to(dev)
    bf = lambda t: t.to(torch.bfloat16).float()
    x = bf(torch.relu(F.conv1d(x, w0, b[0], padding=4, dilation=1)))
    wb = torch.from_numpy(weights["w"].view(np.int16)).to(dev).view(torch.bfloat16).float()   # [5][9][co][ci]
    for l in range(1, 6):
        w = wb[l - 1].permute(1, 2, 0).contiguous()            # [co, ci, 9]
        x = bf(torch.relu(F.conv1d(x, w, b[l], padding=4 * DIL[l], dilation=DIL[l])))
    wo = torch.from_numpy(np.asarray(weights["wout"], np.float32).reshape(-1, CH + 1)).to(dev)   # [heads][129]
    z = x.amax(dim=2) @ wo[:, :CH].T + wo[:, CH]
    return (z[:, 0] if wo.shape[0] == 1 else z).cpu().numpy()


def train(net, X, y, steps: int = 3000, batch: int = 256, lr: float = 1e-3, seed: int = 0):
    import torch
    torch.manual_seed(seed)
    dev = "cuda"
    net = net.to(dev)
    opt = torch.optim.AdamW(net.parameters(), lr=lr, weight_decay=1e-4)
    sched = torch.optim.lr_scheduler.OneCycleLR(opt, max_lr=lr, total_steps=steps, pct_start=0.1)
    pos_w = torch.tensor(max(1.0, float((y == 0).sum()) / max(1.0, float((y == 1).sum()))), device=dev)
    lossf = torch.nn.BCEWithLogitsLoss(pos_weight=pos_w)
    Xd, yd = X.to(dev), torch.from_numpy(y).to(dev)
    g = torch.Generator(device="cpu").manual_seed(seed)
    for it in range(steps):
        idx = torch.randint(0, len(yd), (batch,), generator=g).to(dev)
        with torch.autocast("cuda", dtype=torch.bfloat16):
            out = net(Xd[idx])
        loss = lossf(out.float(), yd[idx])
        opt.zero_grad(set_to_none=True)
        loss.backward()
        torch.nn.utils.clip_grad_norm_(net.parameters(), 1.0)
        opt.step()
        sched.step()
        if it % 500 == 0:
            print(f"step {it} loss {loss.item():.4f}", flush=True)
    return net


def save(weights: dict, path: str, **meta) -> None:
    np.savez_compressed(path, **weights, **{k: np.asarray(v) for k, v in meta.items()})


def load(path: str) -> dict:
    z = np.load(path)
    return {k: z[k] for k in z.files}


class NativeTrainer:
    """The hand-written device trainer (cmgb_filter_trainer_*): the network
    without batch normalisation, trained with AdamW on the GPU; the weights it
    returns load into Prefilter directly."""

    def __init__(self, scanner: "lib.Scanner", W: int, batch: int, seed: int = 0, heads: int = 1):
        import ctypes
        self.lib, self.W, self.B, self.H = scanner.lib, W, batch, heads
        self._h = ctypes.c_void_p()
        err = ctypes.create_string_buffer(256)
        st = self.lib.cmgb_filter_trainer_create_heads(scanner._ctx, W, batch, heads, seed, ctypes.byref(self._h), err)
        if st != 0:
            raise lib.ScanError(st, err.value.decode())

    def close(self):
        if self._h:
            self.lib.cmgb_filter_trainer_destroy(self._h)
            self._h = None

    def set(self, w0, w, bias, wout):
        import ctypes
        arrs = [np.ascontiguousarray(a, np.float32) for a in (w0, w, bias, wout)]
        err = ctypes.create_string_buffer(256)
        st = self.lib.cmgb_filter_trainer_set(self._h, *[a.ctypes.data for a in arrs], err)
        if st != 0:
            raise lib.ScanError(st, err.value.decode())

    def step(self, windows: np.ndarray, labels: np.ndarray, pos_weight, lr: float, weight_decay: float = 1e-4):
        """One batch: windows uint8 [B][2W] residue codes, labels [B] (one
        head) or [B][H]; pos_weight a number or one per head; returns (loss, ms)."""
        import ctypes
        x = np.ascontiguousarray(windows, np.uint8)
        y = np.ascontiguousarray(labels, np.float32)
        assert x.shape == (self.B, 2 * self.W) and y.size == self.B * self.H
        pw = np.ascontiguousarray(np.broadcast_to(np.asarray(pos_weight, np.float32), (self.H,)))
        loss, ms = ctypes.c_float(), ctypes.c_float()
        err = ctypes.create_string_buffer(256)
        st = self.lib.cmgb_filter_trainer_step_heads(self._h, x.ctypes.data, y.ctypes.data, pw.ctypes.data, lr, weight_decay,
                                                     ctypes.byref(loss), ctypes.byref(ms), err)
        if st != 0:
            raise lib.ScanError(st, err.value.decode())
        return loss.value, ms.value

    def get(self, grads: bool = False):
        """fp32 weights (w0 [9,4,128], w [5,9,128,128], bias [6,128], wout [129]), and the last step's gradients."""
        import ctypes
        shapes = [(9, 4, 128), (5, 9, 128, 128), (6, 128), (129,) if self.H == 1 else (self.H, 129)]
        ws = [np.zeros(sh, np.float32) for sh in shapes]
        gs = [np.zeros(sh, np.float32) for sh in shapes] if grads else [None] * 4
        err = ctypes.create_string_buffer(256)
        ptr = [a.ctypes.data if a is not None else None for a in ws + gs]
        st = self.lib.cmgb_filter_trainer_get(self._h, *ptr, err)
        if st != 0:
            raise lib.ScanError(st, err.value.decode())
        return (ws, gs) if grads else ws

    def weights(self) -> dict:
        """The trained network in the layout of export() (BF16 dilated layers)."""
        w0, w, bias, wout = self.get()
        import torch
        wb = torch.from_numpy(w).bfloat16().view(torch.int16).numpy().view(np.uint16)
        return {"w0": w0, "w": wb, "bias": bias, "wout": wout}


# ---------------------------------------------------------------------------
# scan-time use
class Prefilter:
    """The network on one device context (cmgb_filter_*)."""
    LAUNCHES = 7          # kernels per logits() call: layer 0, five convolutions, read-out

    def __init__(self, scanner: "lib.Scanner", weights: dict, W: int):
        self.sc, self.lib = scanner, scanner.lib
        self.W = W
        self.H = int(np.asarray(weights["wout"]).size // 129)       # read-out heads (one per CM)
        self.thr = weights.get("threshold", 0.0)
        self.thr = float(self.thr) if np.ndim(self.thr) == 0 else np.asarray(self.thr, np.float64)
        self.points = weights.get("recall_points")
        self._keep = [np.ascontiguousarray(weights["w0"], np.float32), np.ascontiguousarray(weights["w"], np.uint16),
                      np.ascontiguousarray(weights["bias"], np.float32), np.ascontiguousarray(weights["wout"], np.float32)]
        self._f = ctypes.c_void_p()
        err = ctypes.create_string_buffer(256)
        st = self.lib.cmgb_filter_create_heads(scanner._ctx, W, self.H, *[a.ctypes.data for a in self._keep],
                                               ctypes.byref(self._f), err)
        if st != 0:
            raise lib.ScanError(st, err.value.decode())

    def close(self):
        if self._f:
            self.lib.cmgb_filter_destroy(self._f)
            self._f = ctypes.c_void_p()

    def logits(self, d_dsq_ptr: int, i0: int, j0: int) -> Tuple[np.ndarray, float]:
        """Window logits over [i0, j0] of device-resident residues ([nwin], or
        [nwin][H] for several heads), and the device ms."""
        n = (j0 - i0 + 1 + self.W - 1) // self.W
        out = np.zeros(n * self.H, np.float32)
        nw, ms = ctypes.c_int64(), ctypes.c_float()
        err = ctypes.create_string_buffer(256)
        st = self.lib.cmgb_filter_windows(self.sc._ctx, self._f, d_dsq_ptr, i0, j0, out.ctypes.data, n,
                                          ctypes.byref(nw), ctypes.byref(ms), err)
        if st != 0:
            raise lib.ScanError(st, err.value.decode())
        out = out[: nw.value * self.H]
        return (out if self.H == 1 else out.reshape(nw.value, self.H)), float(ms.value)

    def use_recall(self, recall: float, bits: Optional[float] = None) -> float:
        """Selects the stored validation operating point that keeps this
        fraction of the windows holding a hit of at least `bits` (the bit
        score of E <= 0.01 at the search's size; the largest stored bit level
        not above it, so the recall holds for every such hit); returns its
        threshold.  Files with three columns (recall, threshold, negatives
        kept) store points for one bit level."""
        if self.points is None:
            raise ValueError("the filter file stores no operating points")
        pts = self.points
        if pts.shape[1] >= 5:
            levels = np.unique(pts[:, 0])
            lv = levels[levels <= bits].max() if bits is not None and (levels <= bits).any() else levels.min()
            pts = pts[pts[:, 0] == lv][:, 1:]
        k = int(np.argmin(np.abs(pts[:, 0] - recall)))
        if abs(pts[k, 0] - recall) > 1e-9:
            raise ValueError(f"no stored operating point at recall {recall}")
        self.thr = float(pts[k, 1])
        return self.thr

    def regions(self, logits: np.ndarray, i0: int, j0: int, thr: Optional[float] = None) -> List[Tuple[int, int]]:
        """Kept windows (logit > thr) merged into scan regions [a, b]."""
        thr = self.thr if thr is None else thr
        regs: List[List[int]] = []
        for k in np.nonzero(logits > thr)[0]:
            a, b = i0 + int(k) * self.W, min(j0, i0 + int(k) * self.W + 2 * self.W - 1)
            if regs and a <= regs[-1][1] + 1:
                regs[-1][1] = max(regs[-1][1], b)
            else:
                regs.append([a, b])
        return [(a, b) for a, b in regs]


# ---------------------------------------------------------------------------
# the two pipelines on both strands of one target
def strand_buffer(dsq: np.ndarray) -> np.ndarray:
    """Both strands of a target in one residue buffer: sentinel, top strand
    (L residues), sentinel, reverse complement, sentinel (2L + 3 bytes).
    Strand s's Easel dsq starts at byte s * (L + 1)."""
    L = len(dsq) - 2
    rev = emit.revcomp_dsq(dsq)
    buf = np.empty(2 * L + 3, np.uint8)
    buf[: L + 2] = dsq
    buf[L + 1:] = rev
    return buf


def _ranges_scan(sc: "lib.Scanner", m, d_buf: int, nbuf: int, spans, algo: str, qdb: int, cut: float, stats: dict):
    """One batched launch over sub-ranges of the two-strand buffer; spans are
    (strand, a, b) in strand coordinates; returns per-span hit lists in
    strand coordinates (start, stop, score)."""
    if not spans:
        return []
    L = (nbuf - 3) // 2
    offs = np.array([s * (L + 1) + a - 1 for s, a, b in spans], np.int64)
    lens = np.array([b - a + 1 for s, a, b in spans], np.int64)
    t0 = time.perf_counter()
    rs = sc.scan_batch(m, None, algo=algo, qdbidx=qdb, cutoff=cut, env_cutoff=cut, ranges=(None, offs, lens),
                       device_buf=(d_buf, nbuf))
    stats["wall_ms"][algo] += 1e3 * (time.perf_counter() - t0)
    stats["kernel_ms"][algo] += rs[0].kernel_ms
    stats["launches"] += sc.last_launches()
    stats["calls"][algo] += 1
    h2d, d2h = sc.last_transfer_bytes()
    stats["h2d"] += h2d; stats["d2h"] += d2h
    stats["lengths"][algo] += [int(x) for x in lens]
    return [[(h[0] + a - 1, h[1] + a - 1, h[4]) for h in r.hits] for (s, a, b), r in zip(spans, rs)]


def _new_stats():
    # kernel_ms: device time of each stage's kernels (CUDA events); wall_ms:
    # host wall time of each stage's calls (kernels, copies and the host's
    # hit resolution)
    return {"kernel_ms": {"filter": 0.0, "cyk": 0.0, "inside": 0.0}, "wall_ms": {"filter": 0.0, "cyk": 0.0, "inside": 0.0},
            "launches": 0, "h2d": 0, "d2h": 0, "lengths": {"cyk": [], "inside": []}, "calls": {"cyk": 0, "inside": 0}, "kept": 0}


def _final_stage(sc, m, d_buf, nbuf, cyk_hits, ins_cut, stats):
    """Survivor windows of each strand's CYK hits (pipeline.cyk_windows) and
    the Inside scan of all of them in one launch; hits per strand."""
    from .pipeline import cyk_windows
    L = (nbuf - 3) // 2
    spans = [(s, a, b) for s in (0, 1) for a, b in cyk_windows(cyk_hits[s], m.W, L)]
    out = [[], []]
    for (s, a, b), hs in zip(spans, _ranges_scan(sc, m, d_buf, nbuf, spans, "inside", 2, ins_cut, stats)):
        out[s] += hs
    return out


def filtered_scan(sc: "lib.Scanner", filt: "Prefilter", m, d_buf: int, nbuf: int, cyk_cut: float, ins_cut: float):
    """The learned pipeline over both strands of a target in device memory
    (strand_buffer layout, nbuf bytes at device address d_buf): the filter
    scores every window of each strand, kept windows merge into regions, the
    regions of both strands get the QDB1 CYK scan in one batched launch
    (NULL3, greedy, cutoff cyk_cut), and the survivor windows of the CYK hits
    (padded by W-1 and merged, as the reference pipeline) get the QDB2 Inside
    scan in one more launch.  Returns (hits per strand as (start, stop,
    score) in strand coordinates, statistics)."""
    L = (nbuf - 3) // 2
    st = _new_stats()
    spans = []
    for s in (0, 1):
        t0 = time.perf_counter()
        logit, ms = filt.logits(d_buf + s * (L + 1), 1, L)
        st["kernel_ms"]["filter"] += ms
        st["launches"] += filt.LAUNCHES
        st["d2h"] += 4 * len(logit)
        spans += [(s, a, b) for a, b in filt.regions(logit, 1, L)]
        st["wall_ms"]["filter"] += 1e3 * (time.perf_counter() - t0)
    st["kept"] = sum(b - a + 1 for _, a, b in spans)
    cyk = [[], []]
    for (s, a, b), hs in zip(spans, _ranges_scan(sc, m, d_buf, nbuf, spans, "cyk", 1, cyk_cut, st)):
        cyk[s] += [(h[0], h[1]) for h in hs]
    return _final_stage(sc, m, d_buf, nbuf, cyk, ins_cut, st), st


def plain_scan(sc: "lib.Scanner", m, d_buf: int, nbuf: int, cyk_cut: float, ins_cut: float):
    """The plain GPU pipeline on the same buffer: the single-launch QDB1 CYK
    scan of each whole strand (cmgb_FastCYKScan_dev), then the survivor
    windows of both strands in one batched Inside launch.  The judge of what
    the filter loses.  Returns (hits per strand, statistics)."""
    L = (nbuf - 3) // 2
    st = _new_stats()
    cyk = [[], []]
    for s in (0, 1):
        t0 = time.perf_counter()
        r = sc.scan(m, None, 1, L, algo="cyk", qdbidx=1, cutoff=cyk_cut, env_cutoff=cyk_cut,
                    device_ptr=d_buf + s * (L + 1))
        st["wall_ms"]["cyk"] += 1e3 * (time.perf_counter() - t0)
        st["kernel_ms"]["cyk"] += r.kernel_ms
        st["launches"] += sc.last_launches()
        h2d, d2h = sc.last_transfer_bytes()
        st["h2d"] += h2d; st["d2h"] += d2h
        st["lengths"]["cyk"].append(L)
        st["calls"]["cyk"] += 1
        cyk[s] = [(h[0], h[1]) for h in r.hits]
    st["kept"] = 2 * L
    return _final_stage(sc, m, d_buf, nbuf, cyk, ins_cut, st), st


def _multi_final(sc, models, d_buf, nbuf, cyk_hits, stats):
    """Survivor windows of every (model, strand)'s CYK hits, with each model's
    W, and the Inside scan of all of them in one multi-model launch; hits per
    model and strand."""
    from .pipeline import cyk_windows
    L = (nbuf - 3) // 2
    K = len(models)
    spans = [(k, s, a, b) for k in range(K) for s in (0, 1) for a, b in cyk_windows(cyk_hits[k][s], models[k].W, L)]
    out = [[[], []] for _ in range(K)]
    if not spans:
        return out
    offs = np.array([s * (L + 1) + a - 1 for k, s, a, b in spans], np.int64)
    lens = np.array([b - a + 1 for k, s, a, b in spans], np.int64)
    jobs = [(k, q) for q, (k, s, a, b) in enumerate(spans)]
    rs = sc.scan_multi(models, None, jobs=jobs, algo="inside", qdbidx=2, cutoffs=[INS_CUT] * K, env_cutoff=INS_CUT,
                       ranges=(None, offs, lens), device_buf=(d_buf, nbuf))
    stats["kernel_ms"]["inside"] += rs[0].kernel_ms
    stats["launches"] += sc.last_launches()
    stats["calls"]["inside"] += 1
    h2d, d2h = sc.last_transfer_bytes()
    stats["h2d"] += h2d; stats["d2h"] += d2h
    stats["lengths"]["inside"] += [(k, int(n)) for (k, s, a, b), n in zip(spans, lens)]
    for (k, s, a, b), r in zip(spans, rs):
        out[k][s] += [(h[0] + a - 1, h[1] + a - 1, h[4]) for h in r.hits]
    return out


def filtered_scan_multi(sc: "lib.Scanner", filt: "Prefilter", models, d_buf: int, nbuf: int):
    """The learned pipeline for several CMs over both strands of a target in
    device memory (strand_buffer layout): one pass of the shared trunk gives
    every window one logit per model; each model's kept windows merge into
    its own regions; the QDB1 CYK scan of every (model, region) pair of both
    strands runs in one multi-model launch, and the survivor windows of every
    model in one more (Inside).  Returns (hits [model][strand] as (start,
    stop, score), statistics)."""
    L = (nbuf - 3) // 2
    K = len(models)
    assert filt.H == K
    st = _new_stats()
    spans = []
    for s in (0, 1):
        logit, ms = filt.logits(d_buf + s * (L + 1), 1, L)
        st["kernel_ms"]["filter"] += ms
        st["launches"] += filt.LAUNCHES
        st["d2h"] += 4 * logit.size
        for k in range(K):
            spans += [(k, s, a, b) for a, b in filt.regions(logit[:, k], 1, L, thr=float(filt.thr[k]))]
    st["kept"] = sum(b - a + 1 for _, _, a, b in spans)
    cyk = [[[], []] for _ in range(K)]
    if spans:
        offs = np.array([s * (L + 1) + a - 1 for k, s, a, b in spans], np.int64)
        lens = np.array([b - a + 1 for k, s, a, b in spans], np.int64)
        jobs = [(k, q) for q, (k, s, a, b) in enumerate(spans)]
        rs = sc.scan_multi(models, None, jobs=jobs, algo="cyk", qdbidx=1, cutoffs=[CYK_CUT] * K, env_cutoff=CYK_CUT,
                           ranges=(None, offs, lens), device_buf=(d_buf, nbuf))
        st["kernel_ms"]["cyk"] += rs[0].kernel_ms
        st["launches"] += sc.last_launches()
        st["calls"]["cyk"] += 1
        h2d, d2h = sc.last_transfer_bytes()
        st["h2d"] += h2d; st["d2h"] += d2h
        st["lengths"]["cyk"] += [(k, int(n)) for (k, s, a, b), n in zip(spans, lens)]
        for (k, s, a, b), r in zip(spans, rs):
            cyk[k][s] += [(h[0] + a - 1, h[1] + a - 1) for h in r.hits]
    return _multi_final(sc, models, d_buf, nbuf, cyk, st), st


def plain_scan_multi(sc: "lib.Scanner", models, d_buf: int, nbuf: int):
    """The plain multi-model pipeline on the same buffer: the QDB1 CYK scan of
    both whole strands by every model in one multi-model launch, then every
    model's survivor windows in one Inside launch.  The judge of what the
    several-head filter loses."""
    L = (nbuf - 3) // 2
    K = len(models)
    st = _new_stats()
    offs = np.array([0, L + 1], np.int64)
    lens = np.array([L, L], np.int64)
    jobs = [(k, s) for k in range(K) for s in (0, 1)]
    rs = sc.scan_multi(models, None, jobs=jobs, algo="cyk", qdbidx=1, cutoffs=[CYK_CUT] * K, env_cutoff=CYK_CUT,
                       ranges=(None, offs, lens), device_buf=(d_buf, nbuf))
    st["kernel_ms"]["cyk"] += rs[0].kernel_ms
    st["launches"] += sc.last_launches()
    st["calls"]["cyk"] += 1
    st["lengths"]["cyk"] += [(k, L) for k, s in jobs]
    cyk = [[[], []] for _ in range(K)]
    for (k, s), r in zip(jobs, rs):
        cyk[k][s] = [(h[0], h[1]) for h in r.hits]
    st["kept"] = 2 * L * K
    return _multi_final(sc, models, d_buf, nbuf, cyk, st), st


def _windows_job(args):
    name, n, seed, first = args
    m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", f"{name}.model.npz"))
    return make_windows(m, n, np.random.default_rng(seed), first)


def make_windows_parallel(name: str, n: int, seed: int, procs: int = 0) -> List[np.ndarray]:
    """make_windows over worker processes (spawned: call before any GPU use)."""
    import multiprocessing as mp
    procs = procs or max(1, min(16, os.cpu_count() or 1))
    per = (n + procs - 1) // procs
    jobs = [(name, min(per, n - k * per), seed * 1000 + k, k * per) for k in range(procs) if k * per < n]
    with mp.get_context("spawn").Pool(len(jobs)) as pool:
        parts = pool.map(_windows_job, jobs)
    return [w for p in parts for w in p]


def train_native(sc, W: int, wins: List[np.ndarray], y: np.ndarray, steps: int, batch: int = 256,
                 lr: float = 1e-3, seed: int = 0) -> dict:
    """Trains the network (no batch normalisation) with the device trainer:
    batches drawn uniformly from wins (Easel dsq windows of 2W residues, or
    an array [n][2W] of residue codes),
    positive class weighted by the class ratio, learning rate warmed up over
    the first 10% of steps and annealed by a cosine; returns the weights."""
    rng = np.random.default_rng(seed)
    X = wins if isinstance(wins, np.ndarray) else np.stack([w[1:-1] for w in wins]).astype(np.uint8)
    posw = max(1.0, float((y == 0).sum()) / max(1.0, float((y == 1).sum())))
    tr = NativeTrainer(sc, W, batch, seed=seed + 1)
    try:
        for it in range(steps):
            idx = rng.integers(0, len(X), batch)
            warm = max(1, steps // 10)
            f = (it + 1) / warm if it < warm else 0.5 * (1 + np.cos(np.pi * (it - warm) / max(1, steps - warm)))
            loss, ms = tr.step(X[idx], y[idx].astype(np.float32), posw, lr * f)
            if it % 500 == 0:
                print(f"step {it} loss {loss:.4f} ({ms:.1f} ms)", flush=True)
        return tr.weights()
    finally:
        tr.close()


def train_bulk(name: str, out: str, nwin: int, epochs: float, nval: int = 60000, seed: int = 20261206,
               batch: int = 256, lr: float = 1e-3) -> None:
    """The bulk recipe: nwin training windows (emitted / iid / shuffled,
    make_window_block), labelled by the plain scan's final-stage score
    (positive: a final hit of at least INS_CUT bits), trained with the
    device trainer for `epochs` passes, operating points from nval fresh
    validation windows scored by the inference kernels."""
    t0 = time.time()
    m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", f"{name}.model.npz"))
    block = make_window_block_parallel(name, nwin, seed)            # before the first GPU call
    vblock = make_window_block_parallel(name, nval, seed + 1)
    print(f"{nwin} + {nval} windows made in {time.time() - t0:.0f}s", flush=True)
    sc = lib.Scanner(0)
    sc.autotune(m, 1, "cyk"); sc.autotune(m, 2, "inside")
    kinds = np.arange(nwin) % 3
    best = best_inside_scores(sc, m, block, rows=np.nonzero(kinds != 1)[0])   # iid windows: no hit assumed
    vbest = best_inside_scores(sc, m, vblock)
    y = (best >= INS_CUT).astype(np.float32)
    print(f"labelled in {time.time() - t0:.0f}s: {int(y.sum())} positive; validation: {int((vbest >= INS_CUT).sum())} "
          f"positive, {int(np.isfinite(vbest[np.arange(nval) % 3 == 1]).sum())} iid windows with a hit", flush=True)
    steps = int(epochs * nwin / batch)
    wts = train_native(sc, m.W, block[:, 1:-1], y, steps, batch=batch, lr=lr)
    print(f"trained {steps} steps in {time.time() - t0:.0f}s", flush=True)
    f = Prefilter(sc, wts, m.W)
    vl = block_logits(f, vblock)
    f.close()
    pts = operating_points(vl, vbest, np.arange(nval) % 3 == 1)
    for r in pts:
        print(f"  bits {r[0]:5.1f} recall {r[1]:.3f}: threshold {r[2]:8.3f}, negatives kept {r[3]:.4f}, "
              f"background kept {r[4]:.4f}", flush=True)
    thr = float(pts[(pts[:, 0] == 17.2) & (pts[:, 1] == 0.99)][0, 2])
    save(wts, out, threshold=thr, W=m.W, trained_windows=nwin, recall_points=pts,
         trainer=np.array("cmgb_filter_trainer (device, no batch normalisation)"),
         recipe=np.array(f"prefilter.train_bulk({name!r}, nwin={nwin}, epochs={epochs}, nval={nval}, seed={seed}, "
                         f"batch={batch}, lr={lr})"))
    sc.close()
    print(f"saved {out} after {time.time() - t0:.0f}s", flush=True)


def main(argv):
    if len(argv) >= 4 and argv[1] == "train-bulk-multi":
        train_bulk_multi(argv[2].split(","), argv[3], int(argv[4]) if len(argv) > 4 else 300000,
                         float(argv[5]) if len(argv) > 5 else 2.0)
        return 0
    if len(argv) >= 4 and argv[1] == "train-bulk":
        train_bulk(argv[2], argv[3], int(argv[4]) if len(argv) > 4 else 600000, float(argv[5]) if len(argv) > 5 else 2.0)
        return 0
    if len(argv) < 4 or argv[1] not in ("train", "train-native"):
        print(__doc__)
        return 2
    import torch
    native = argv[1] == "train-native"
    name, out = argv[2], argv[3]
    nwin = int(argv[4]) if len(argv) > 4 else 60000
    steps = int(argv[5]) if len(argv) > 5 else 4000
    m = cmfile.load_npz(os.path.join(ROOT, "tests", "golden", f"{name}.model.npz"))
    t0 = time.time()
    wins = make_windows_parallel(name, nwin, 20261205)       # before the first GPU call
    sc = lib.Scanner(0)
    y = label_windows(sc, m, wins)
    print(f"{nwin} windows, {int(y.sum())} positive, made+labelled in {time.time() - t0:.0f}s", flush=True)
    ntr = int(0.85 * nwin)
    if native:
        wts = train_native(sc, m.W, wins[:ntr], y[:ntr], steps)
    else:
        X = onehot(wins)
        net = train(make_net(), X[:ntr], y[:ntr], steps=steps)
        wts = export(net.float())
    # threshold: keep >= 99% of the validation windows holding a hit with
    # E <= 0.01 at 4 Mb per search (E_BITS, from the CM's ECMLI calibration):
    # the loss budget of at most 1% of those hits
    val = reference_logits(wts, wins[ntr:])
    best = label_windows.best[ntr:]
    print(f"validation: {int((y[ntr:] == 1).sum())} positives, {int((best >= E_BITS).sum())} with E <= 0.01", flush=True)
    pos = np.sort(val[best >= E_BITS])
    thr = float(pos[int(0.01 * len(pos))] - 1e-3) if len(pos) else 0.0
    kept_neg = float((val[y[ntr:] == 0] > thr).mean())
    print(f"threshold {thr:.3f}: validation positives kept {(val[y[ntr:] == 1] > thr).mean():.4f}, "
          f"negatives kept {kept_neg:.4f}", flush=True)
    bg = np.array([k % 3 == 1 for k in range(ntr, nwin)])      # pure background windows
    print(f"  background windows kept {float((val[bg] > thr).mean()):.4f}", flush=True)
    points = []                 # operating points: (recall of E <= 0.01 windows, threshold, negatives kept)
    for q in (0.9, 0.95, 0.98, 0.99, 0.995, 0.999):
        t = float(pos[int((1 - q) * len(pos))] - 1e-3) if len(pos) else 0.0
        nk = float((val[y[ntr:] == 0] > t).mean())
        points.append((q, t, nk))
        print(f"  recall {q}: threshold {t:.3f}, negatives kept {nk:.4f}", flush=True)
    save(wts, out, threshold=thr, W=m.W, trained_windows=ntr, recall_points=np.array(points),
         trainer=np.array("cmgb_filter_trainer (device, no batch normalisation)" if native else "PyTorch (batch normalisation folded)"))
    sc.close()
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv))
