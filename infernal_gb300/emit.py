"""Sampling sequences from a CM and building seeded synthetic targets.

``sample`` draws one sequence from a CM's generative model (a parse tree
walk: start at ROOT_S, emit by state type, follow transitions, split at
bifurcations), the method of Infernal's EmitParsetree (src/cm_parsetree.c:1890).
It uses the unconfigured (global) probabilities of :func:`cmfile.read_cm`.

``make_target`` builds an iid background of a given GC content with emitted
sequences embedded at seeded positions on random strands; the stand-in for
the synthetic targets of the benchmark configurations.
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np

from . import cmfile as cf

_COMP = str.maketrans("ACGU", "UGCA")


def revcomp(s: str) -> str:
    return s.translate(_COMP)[::-1]


def sample(m: cf.CMModel, rng: np.random.Generator, max_len: int = 100000) -> str:
    """One sequence emitted by CM m in global mode (its transitions before
    local configuration, ``m.t_global``)."""
    K = m.K
    alph = "ACGU"
    out_left: List[str] = []

    def walk(v: int) -> str:
        parts_l: List[str] = []
        parts_r: List[str] = []
        while True:
            st = int(m.sttype[v])
            if st == cf.E_st:
                return "".join(parts_l) + "".join(reversed(parts_r))
            if st == cf.B_st:
                left = walk(int(m.cfirst[v]))
                right = walk(int(m.cnum[v]))
                return "".join(parts_l) + left + right + "".join(reversed(parts_r))
            if st == cf.MP_st:
                p = m.e[v, : K * K].astype(np.float64)
                x = rng.choice(K * K, p=p / p.sum())
                parts_l.append(alph[x // K]); parts_r.append(alph[x % K])
            elif st in (cf.ML_st, cf.IL_st):
                p = m.e[v, :K].astype(np.float64)
                parts_l.append(alph[rng.choice(K, p=p / p.sum())])
            elif st in (cf.MR_st, cf.IR_st):
                p = m.e[v, :K].astype(np.float64)
                parts_r.append(alph[rng.choice(K, p=p / p.sum())])
            n = int(m.cnum[v])
            t = (m.t_global if m.t_global is not None else m.t)[v, :n].astype(np.float64)
            v = int(m.cfirst[v]) + int(rng.choice(n, p=t / t.sum()))
            if len(parts_l) + len(parts_r) > max_len:
                raise RuntimeError("runaway emission")

    return walk(0)


class Sampler:
    """The same generative walk as :func:`sample`, from per-state cumulative
    emission and transition tables drawn with a ``random.Random`` stream:
    about fifty times faster, for bulk training data.  (Its random stream is
    not ``sample``'s: the two give different sequences for one seed.)"""

    def __init__(self, m: cf.CMModel):
        import bisect
        self._bisect = bisect.bisect_right
        K = m.K
        T = m.t_global if m.t_global is not None else m.t
        self.st = [int(x) for x in m.sttype]
        self.cf = [int(x) for x in m.cfirst]
        self.cn = [int(x) for x in m.cnum]
        self.ecum, self.tcum = [], []
        for v in range(m.M):
            st = self.st[v]
            if st == cf.MP_st:
                p = m.e[v, : K * K].astype(np.float64)
            elif st in (cf.ML_st, cf.IL_st, cf.MR_st, cf.IR_st):
                p = m.e[v, :K].astype(np.float64)
            else:
                p = None
            self.ecum.append(list(np.cumsum(p / p.sum())) if p is not None else None)
            if st in (cf.E_st, cf.B_st):
                self.tcum.append(None)
            else:
                t = T[v, : self.cn[v]].astype(np.float64)
                self.tcum.append(list(np.cumsum(t / t.sum())))

    def _pick(self, cum, u):
        k = self._bisect(cum, u)
        return k if k < len(cum) else len(cum) - 1

    def sample(self, rnd, max_len: int = 100000) -> str:
        alph = "ACGU"
        st, cfr, cn, ecum, tcum, pick = self.st, self.cf, self.cn, self.ecum, self.tcum, self._pick

        def walk(v: int) -> str:
            left: List[str] = []
            right: List[str] = []
            while True:
                t = st[v]
                if t == cf.E_st:
                    return "".join(left) + "".join(reversed(right))
                if t == cf.B_st:
                    return "".join(left) + walk(cfr[v]) + walk(cn[v]) + "".join(reversed(right))
                if t == cf.MP_st:
                    x = pick(ecum[v], rnd.random())
                    left.append(alph[x // 4]); right.append(alph[x % 4])
                elif t == cf.ML_st or t == cf.IL_st:
                    left.append(alph[pick(ecum[v], rnd.random())])
                elif t == cf.MR_st or t == cf.IR_st:
                    right.append(alph[pick(ecum[v], rnd.random())])
                v = cfr[v] + pick(tcum[v], rnd.random())
                if len(left) + len(right) > max_len:
                    raise RuntimeError("runaway emission")

        return walk(0)


def background(rng: np.random.Generator, L: int, gc: float) -> np.ndarray:
    """iid residues (digital codes 0..3) with P(G)=P(C)=gc/2."""
    p = np.array([(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2])
    return rng.choice(4, size=L, p=p).astype(np.uint8)


def make_target(rng: np.random.Generator, L: int, gc, inserts: List[str],
                seg_len: int = 50_000) -> Tuple[np.ndarray, List[tuple]]:
    """Digital target (Easel dsq with sentinels) of length L: iid background
    with each insert written over it at a random non-overlapping position on a
    random strand.  gc is one GC fraction, or a (low, high) range: then every
    segment of seg_len residues draws its own GC fraction uniformly from it.
    Returns (dsq, [(start, stop, strand)])."""
    if isinstance(gc, tuple):
        parts, left = [], L
        while left > 0:
            n = min(seg_len, left)
            parts.append(background(rng, n, float(rng.uniform(gc[0], gc[1]))))
            left -= n
        seq = np.concatenate(parts)
    else:
        seq = background(rng, L, gc)
    spans = []
    if inserts:
        slots = np.sort(rng.choice(max(1, L // 2000), size=min(len(inserts), max(1, L // 2000)), replace=False))
        for k, ins in zip(slots, inserts):
            s = ins if rng.random() < 0.5 else revcomp(ins)
            start = int(k) * 2000 + int(rng.integers(0, max(1, 2000 - len(s))))
            if start + len(s) > L:
                continue
            seq[start: start + len(s)] = np.frombuffer(s.encode().translate(bytes.maketrans(b"ACGU", b"\x00\x01\x02\x03")), np.uint8)
            spans.append((start + 1, start + len(s), "+" if s is ins else "-"))
    dsq = np.empty(L + 2, np.uint8)
    dsq[0] = dsq[-1] = cf.DSQ_SENTINEL
    dsq[1:-1] = seq
    return dsq, spans


def revcomp_dsq(dsq: np.ndarray) -> np.ndarray:
    """Reverse complement of a canonical-residue digital sequence."""
    out = dsq.copy()
    body = dsq[1:-1][::-1]
    comp = np.array([3, 2, 1, 0] + list(range(4, 256)), np.uint8)
    out[1:-1] = comp[body]
    return out
