"""Infernal 1.1 ASCII CM reader and search configuration (host side).

Reads a ``.cm`` file in the INFERNAL1/a format (``src/cm_file.c:1539-2121``,
state-line grammar ``:1963-2040``) and configures it the way ``cm_Configure``
does for a scan (``src/cm_modelconfig.c:139-373``): renormalisation
(``src/cm.c:344``), local begins/ends (``cm_localize``,
``src/cm_modelconfig.c:467``), and log-odds conversion (``CMLogoddsify``,
``src/cm.c:784-935``; optimised emission tables ``FCalcOptimizedEmitScores``
``src/cm.c:3604`` and ``ICopyOptimizedEmitScoresFromFloats`` ``src/cm.c:3855``).

The C code mixes float and double arithmetic; every step below keeps the same
precision at the same point (numpy float32 scalars for C ``float``, Python
floats for C ``double``, ``math.log``/``math.exp`` for libm) so that the
score tables come out bit-identical to the C expressions they restate.

The result is a :class:`CMModel` holding flat numpy arrays in the layout of
``cmgb_model_desc`` (``include/infernal_gb300.h``).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

f32 = np.float32

# ---- constants (src/infernal.h:148-243) ------------------------------------
IMPOSSIBLE = -1e36
INFTY = 987654321
INTSCALE = f32(1000.0)
MAXCONNECT = 6

D_st, MP_st, ML_st, MR_st, IL_st, IR_st, S_st, E_st, B_st, EL_st = range(10)
STATECODE = {"D": D_st, "MP": MP_st, "ML": ML_st, "MR": MR_st, "IL": IL_st,
             "IR": IR_st, "S": S_st, "E": E_st, "B": B_st, "EL": EL_st}
BIF_nd, MATP_nd, MATL_nd, MATR_nd, BEGL_nd, BEGR_nd, ROOT_nd, END_nd = range(8)
NODECODE = {"BIF": BIF_nd, "MATP": MATP_nd, "MATL": MATL_nd, "MATR": MATR_nd,
            "BEGL": BEGL_nd, "BEGR": BEGR_nd, "ROOT": ROOT_nd, "END": END_nd}
(ROOT_S, ROOT_IL, ROOT_IR, BEGL_S, BEGR_S, BEGR_IL, MATP_MP, MATP_ML, MATP_MR,
 MATP_D, MATP_IL, MATP_IR, MATL_ML, MATL_D, MATL_IL, MATR_MR, MATR_D, MATR_IR,
 END_E, BIF_B, END_EL) = range(21)

# DeriveUniqueStateCode (src/cm.c): (node type, state type) -> unique id
_STID = {
    (ROOT_nd, S_st): ROOT_S, (ROOT_nd, IL_st): ROOT_IL, (ROOT_nd, IR_st): ROOT_IR,
    (BEGL_nd, S_st): BEGL_S, (BEGR_nd, S_st): BEGR_S, (BEGR_nd, IL_st): BEGR_IL,
    (MATP_nd, MP_st): MATP_MP, (MATP_nd, ML_st): MATP_ML, (MATP_nd, MR_st): MATP_MR,
    (MATP_nd, D_st): MATP_D, (MATP_nd, IL_st): MATP_IL, (MATP_nd, IR_st): MATP_IR,
    (MATL_nd, ML_st): MATL_ML, (MATL_nd, D_st): MATL_D, (MATL_nd, IL_st): MATL_IL,
    (MATR_nd, MR_st): MATR_MR, (MATR_nd, D_st): MATR_D, (MATR_nd, IR_st): MATR_IR,
    (END_nd, E_st): END_E, (BIF_nd, B_st): BIF_B,
}

# ---- RNA alphabet (Easel eslRNA) --------------------------------------------
RNA_SYM = "ACGU-RYMKSWHBVDN*~"
K_RNA, KP_RNA = 4, 18
_DEGEN = ["A", "C", "G", "U", "", "AG", "CU", "AC", "GU", "CG", "AU", "ACU",
          "CGU", "ACG", "AGU", "ACGU", "", ""]
DEGEN = [[("ACGU"[y] in _DEGEN[x]) for y in range(4)] for x in range(18)]
NDEGEN = [sum(r) for r in DEGEN]
DSQ_SENTINEL = 255

_DIGI = {c: i for i, c in enumerate(RNA_SYM)}
_DIGI.update({"T": 3, "X": 15, ".": 4, "_": 4})


def digitize(seq: str) -> np.ndarray:
    """Easel-style digital sequence: dsq[0] and dsq[L+1] are sentinels,
    dsq[1..L] are residue codes of the RNA alphabet (T is read as U)."""
    out = np.empty(len(seq) + 2, dtype=np.uint8)
    out[0] = out[-1] = DSQ_SENTINEL
    s = seq.upper()
    try:
        out[1:-1] = np.frombuffer(bytes(_DIGI[c] for c in s), dtype=np.uint8)
    except KeyError as e:  # pragma: no cover - input error path
        raise ValueError(f"invalid residue {e.args[0]!r} for the RNA alphabet") from None
    return out


def read_fasta(path: str) -> List[tuple]:
    """Returns [(name, sequence_string)] for a FASTA file."""
    recs, name, buf = [], None, []
    with open(path) as fh:
        for line in fh:
            line = line.strip()
            if not line:
                continue
            if line.startswith(">"):
                if name is not None:
                    recs.append((name, "".join(buf)))
                name, buf = line[1:].split()[0] if len(line) > 1 else "", []
            else:
                buf.append(line)
    if name is not None:
        recs.append((name, "".join(buf)))
    return recs


# ---- C arithmetic helpers ---------------------------------------------------
def sreLOG2(x) -> float:
    """src/infernal.h:153 ``((x) > 0 ? log(x) * 1.44269504 : IMPOSSIBLE)`` (double)."""
    x = float(x)
    return math.log(x) * 1.44269504 if x > 0 else IMPOSSIBLE


def sreEXP2(x) -> float:
    """src/infernal.h:154 (double)."""
    return math.exp(float(x) * 0.69314718)


def ascii2prob(tok: str, null) -> np.float32:
    """src/cm_file.c:3353: ``exp(atof(s)/1.44269504)*null`` returned as float."""
    if tok.startswith("*"):
        return f32(0.0)
    return f32(math.exp(float(tok) / 1.44269504) * float(f32(null)))


def Prob2Score(p, null) -> int:
    """src/cm.c:4201: ``(int) floor(0.5 + INTSCALE * sreLOG2(p/null))``; the
    quotient p/null is a float division."""
    p = f32(p)
    if p == 0.0:
        return -INFTY
    q = f32(p / f32(null))
    return int(math.floor(0.5 + float(INTSCALE) * sreLOG2(q)))


def fsum_kahan(v) -> np.float32:
    """Easel's compensated float vector sum."""
    s, c = f32(0.0), f32(0.0)
    for x in v:
        y = f32(f32(x) - c)
        t = f32(s + y)
        c = f32(f32(t - s) - y)
        s = t
    return s


def fnorm(v: np.ndarray) -> None:
    """esl_vec_FNorm in place (float32)."""
    s = fsum_kahan(v)
    if s != 0.0:
        for i in range(len(v)):
            v[i] = f32(v[i] / s)
    else:
        v[:] = f32(1.0) / f32(len(v))


# ---- the model ---------------------------------------------------------------
@dataclass
class CMModel:
    name: str
    M: int
    nodes: int
    clen: int
    W: int
    K: int = K_RNA
    Kp: int = KP_RNA
    header: Dict[str, str] = field(default_factory=dict)
    sttype: np.ndarray = None
    stid: np.ndarray = None
    ndidx: np.ndarray = None
    cfirst: np.ndarray = None
    cnum: np.ndarray = None
    plast: np.ndarray = None
    pnum: np.ndarray = None
    ndtype: np.ndarray = None
    nodemap: np.ndarray = None
    dmin1: np.ndarray = None
    dmax1: np.ndarray = None
    dmin2: np.ndarray = None
    dmax2: np.ndarray = None
    t: np.ndarray = None          # [M, 6] float32 probabilities
    t_global: np.ndarray = None   # [M, 6] transitions before local configuration
    e: np.ndarray = None          # [M, K*K] float32 probabilities
    null: np.ndarray = None       # [K] float32
    begin: np.ndarray = None
    end: np.ndarray = None
    el_selfsc: np.float32 = f32(0.0)
    null3_omega: np.float32 = f32(0.0)
    pbegin: np.float32 = f32(0.05)
    pend: np.float32 = f32(0.05)
    flags: int = 0
    # configured scores
    tsc: np.ndarray = None
    itsc: np.ndarray = None
    oesc: np.ndarray = None
    ioesc: np.ndarray = None
    endsc: np.ndarray = None
    beginsc: np.ndarray = None
    iendsc: np.ndarray = None
    ibeginsc: np.ndarray = None
    iel_selfsc: int = 0
    lmesc: np.ndarray = None
    rmesc: np.ndarray = None
    ilmesc: np.ndarray = None
    irmesc: np.ndarray = None
    # truncated scanning (truncation_tables)
    emap_lpos: np.ndarray = None
    emap_rpos: np.ndarray = None
    tr_g_pty: np.ndarray = None
    tr_l_pty: np.ndarray = None
    tr_ig_pty: np.ndarray = None
    tr_il_pty: np.ndarray = None
    configured: bool = False
    ecm: Dict[str, tuple] = field(default_factory=dict)

    # -- derived helpers
    def bands(self, qdbidx: int):
        """dmin/dmax of band set qdbidx (0 = no bands)."""
        if qdbidx == 1:
            return self.dmin1, self.dmax1
        if qdbidx == 2:
            return self.dmin2, self.dmax2
        return None, None


def read_cm(path: str, which: int = 0) -> CMModel:
    """Parses the ``which``-th model of an INFERNAL1/a CM file
    (src/cm_file.c:1539 read_asc_1p1_cm).  The filter HMM that follows each
    CM is skipped."""
    with open(path) as fh:
        lines = fh.read().split("\n")
    idx, model_no = 0, -1
    while idx < len(lines):
        if lines[idx].startswith("INFERNAL1/a"):
            model_no += 1
            if model_no == which:
                break
        idx += 1
    else:
        raise ValueError(f"{path}: model {which} not found")
    idx += 1
    hdr: Dict[str, str] = {}
    while idx < len(lines) and lines[idx].strip() != "CM":
        ln = lines[idx]
        if ln.strip():
            tag, _, rest = ln.partition(" ")
            hdr[tag] = rest.strip()
        idx += 1
    idx += 1
    M = int(hdr["STATES"])
    nodes = int(hdr["NODES"])
    m = CMModel(name=hdr.get("NAME", "?"), M=M, nodes=nodes, clen=int(hdr["CLEN"]),
                W=int(hdr["W"]), header=hdr)
    if hdr.get("ALPH", "RNA") != "RNA":
        raise ValueError("only the RNA alphabet is supported")
    K = m.K
    m.pbegin = f32(float(hdr.get("PBEGIN", "0.05")))
    m.pend = f32(float(hdr.get("PEND", "0.05")))
    m.el_selfsc = f32(float(hdr["ELSELF"]))
    m.null3_omega = f32(float(hdr.get("N3OMEGA", str(2.0 ** -16))))
    for tag in ("ECMLC", "ECMGC", "ECMLI", "ECMGI"):
        if tag in hdr:
            m.ecm[tag] = tuple(float(x) for x in hdr[tag].split())
    null = np.array([ascii2prob(tok, 1.0 / K) for tok in hdr["NULL"].split()[:K]], dtype=np.float32)
    m.null = null
    m.sttype = np.zeros(M, np.int8)
    m.stid = np.zeros(M, np.int8)
    m.ndidx = np.zeros(M, np.int32)
    m.cfirst = np.zeros(M, np.int32)
    m.cnum = np.zeros(M, np.int32)
    m.plast = np.zeros(M, np.int32)
    m.pnum = np.zeros(M, np.int32)
    m.ndtype = np.zeros(nodes, np.int8)
    m.nodemap = np.zeros(nodes, np.int32)
    for a in ("dmin1", "dmax1", "dmin2", "dmax2"):
        setattr(m, a, np.zeros(M, np.int32))
    m.t = np.zeros((M, MAXCONNECT), np.float32)
    m.e = np.zeros((M, K * K), np.float32)
    nd = -1
    v = 0
    while v < M:
        ln = lines[idx]
        idx += 1
        toks = ln.split()
        if not toks:
            continue
        if toks[0] == "[":
            nd = int(toks[2])
            m.ndtype[nd] = NODECODE[toks[1]]
            m.nodemap[nd] = v
            continue
        st = STATECODE[toks[0]]
        if int(toks[1]) != v:
            raise ValueError(f"state index mismatch at {v}")
        m.sttype[v] = st
        m.plast[v], m.pnum[v] = int(toks[2]), int(toks[3])
        m.cfirst[v], m.cnum[v] = int(toks[4]), int(toks[5])
        m.dmin2[v], m.dmin1[v], m.dmax1[v], m.dmax2[v] = (int(x) for x in toks[6:10])
        p = 10
        if st != B_st:
            for x in range(m.cnum[v]):
                m.t[v, x] = ascii2prob(toks[p], 1.0)
                p += 1
        if st in (ML_st, MR_st, IL_st, IR_st):
            for x in range(K):
                m.e[v, x] = ascii2prob(toks[p], m.null[x])
                p += 1
        elif st == MP_st:
            for x in range(K):
                for y in range(K):
                    m.e[v, x * K + y] = ascii2prob(toks[p], f32(m.null[x] * m.null[y]))
                    p += 1
        m.ndidx[v] = nd
        m.stid[v] = _STID[(int(m.ndtype[nd]), st)]
        v += 1
    _renormalize(m)
    m.t_global = m.t.copy()
    return m


def _renormalize(m: CMModel) -> None:
    """CMRenormalize (src/cm.c:344-375)."""
    fnorm(m.null)
    for v in range(m.M):
        st = m.sttype[v]
        if m.cnum[v] > 0 and st != B_st:
            row = m.t[v, : m.cnum[v]].copy()
            fnorm(row)
            m.t[v, : m.cnum[v]] = row
        if st in (ML_st, MR_st, IL_st, IR_st):
            row = m.e[v, : m.K].copy()
            fnorm(row)
            m.e[v, : m.K] = row
        elif st == MP_st:
            row = m.e[v, : m.K * m.K].copy()
            fnorm(row)
            m.e[v, :] = row


def _localize(m: CMModel) -> None:
    """cm_localize + cm_CalculateLocalBeginProbs (src/cm_modelconfig.c:397-560)."""
    internal = (MATP_nd, MATL_nd, MATR_nd, BIF_nd)
    nstarts = sum(1 for nd in range(2, m.nodes) if m.ndtype[nd] in internal)
    m.begin = np.zeros(m.M, np.float32)
    m.begin[m.nodemap[1]] = f32(1.0 - float(m.pbegin))
    p = f32(m.pbegin / f32(nstarts))
    for nd in range(2, m.nodes):
        if m.ndtype[nd] in internal:
            m.begin[m.nodemap[nd]] = p
    m.t[0, : m.cnum[0]] = 0.0
    exits = (MATP_nd, MATL_nd, MATR_nd, BEGL_nd, BEGR_nd)
    nexits = sum(1 for nd in range(1, m.nodes)
                 if m.ndtype[nd] in exits and m.ndtype[nd + 1] != END_nd)
    m.end = np.zeros(m.M, np.float32)
    for nd in range(1, m.nodes):
        if m.ndtype[nd] in exits and m.ndtype[nd + 1] != END_nd:
            v = m.nodemap[nd]
            m.end[v] = f32(m.pend / f32(nexits))
            denom = fsum_kahan(m.t[v, : m.cnum[v]])
            denom = f32(denom + m.end[v])
            scale = f32(1.0 / float(denom))
            for x in range(m.cnum[v]):
                m.t[v, x] = f32(m.t[v, x] * scale)
    m.flags |= 1 | 2  # CMGB_LOCAL_BEGIN | CMGB_LOCAL_END


def _favg_score(a: int, sc) -> np.float32:
    """Average score of the canonical residues a degenerate code stands for
    (Easel esl_abc_FAvgScore)."""
    if a < K_RNA:
        return f32(sc[a])
    if NDEGEN[a] == 0:
        return f32(0.0)
    r = f32(0.0)
    for i in range(K_RNA):
        if DEGEN[a][i]:
            r = f32(r + f32(sc[i]))
    return f32(r / f32(NDEGEN[a]))


def _fcount(a: int) -> np.ndarray:
    """Easel esl_abc_FCount of one residue with weight 1 into a zero vector."""
    v = np.zeros(K_RNA, np.float32)
    if a < K_RNA:
        v[a] = 1.0
    elif NDEGEN[a] > 0:
        for i in range(K_RNA):
            if DEGEN[a][i]:
                v[i] = f32(v[i] + f32(f32(1.0) / f32(NDEGEN[a])))
    return v


def _fexpect_sc_vec(sc: np.ndarray, null: np.ndarray) -> None:
    """Easel esl_abc_FExpectScVec: fill degenerate entries with the
    background-weighted expected score of the residues they stand for."""
    for x in range(K_RNA + 1, KP_RNA - 2):
        result, denom = f32(0.0), f32(0.0)
        for i in range(K_RNA):
            if DEGEN[x][i]:
                result = f32(result + f32(sc[i] * null[i]))
                denom = f32(denom + null[i])
        sc[x] = f32(result / denom) if denom != 0.0 else f32(0.0)


def _iexpect_sc_vec(sc: np.ndarray, null: np.ndarray) -> None:
    """Easel esl_abc_IExpectScVec (integer scores, float accumulation)."""
    for x in range(K_RNA + 1, KP_RNA - 2):
        result, denom = f32(0.0), f32(0.0)
        for i in range(K_RNA):
            if DEGEN[x][i]:
                result = f32(result + f32(f32(sc[i]) * null[i]))
                denom = f32(denom + null[i])
        sc[x] = int(result / denom) if denom != 0.0 else 0


def configure(m: CMModel, local: bool = True) -> CMModel:
    """cm_Configure for a scan: localise (default search mode) and compute
    log-odds score tables (CMLogoddsify, src/cm.c:784-935)."""
    if m.configured:
        return m
    M, K, Kp = m.M, m.K, m.Kp
    if local:
        _localize(m)
    else:
        m.begin = np.zeros(M, np.float32)
        m.end = np.zeros(M, np.float32)
    if float(f32(m.el_selfsc * f32(m.W))) < IMPOSSIBLE:
        m.el_selfsc = f32(IMPOSSIBLE / (m.W + 1))
    m.tsc = np.full((M, MAXCONNECT), f32(0.0), np.float32)
    m.itsc = np.zeros((M, MAXCONNECT), np.int32)
    esc = np.zeros((M, K * K), np.float32)
    iesc = np.zeros((M, K * K), np.int32)
    m.lmesc = np.zeros((M, Kp), np.float32)
    m.rmesc = np.zeros((M, Kp), np.float32)
    m.ilmesc = np.zeros((M, Kp), np.int32)
    m.irmesc = np.zeros((M, Kp), np.int32)
    m.beginsc = np.zeros(M, np.float32)
    m.endsc = np.zeros(M, np.float32)
    m.ibeginsc = np.zeros(M, np.int32)
    m.iendsc = np.zeros(M, np.int32)
    null = m.null
    for v in range(M):
        st = m.sttype[v]
        for arr, ia in ((m.lmesc, m.ilmesc), (m.rmesc, m.irmesc)):
            arr[v, K] = arr[v, Kp - 2] = arr[v, Kp - 1] = f32(IMPOSSIBLE)
            ia[v, K] = ia[v, Kp - 2] = ia[v, Kp - 1] = -INFTY
        if st != B_st and st != E_st:
            for x in range(m.cnum[v]):
                m.tsc[v, x] = f32(sreLOG2(m.t[v, x]))
                m.itsc[v, x] = Prob2Score(m.t[v, x], 1.0)
        if st == MP_st:
            lm = np.zeros(K, np.float32)
            rm = np.zeros(K, np.float32)
            for x in range(K):
                for y in range(K):
                    nn = f32(null[x] * null[y])
                    esc[v, x * K + y] = f32(sreLOG2(f32(m.e[v, x * K + y] / nn)))
                    iesc[v, x * K + y] = Prob2Score(m.e[v, x * K + y], nn)
                    lm[x] = f32(lm[x] + m.e[v, x * K + y])
                    rm[y] = f32(rm[y] + m.e[v, x * K + y])
            for x in range(K):
                m.ilmesc[v, x] = Prob2Score(lm[x], null[x])
                m.irmesc[v, x] = Prob2Score(rm[x], null[x])
                m.lmesc[v, x] = f32(sreLOG2(f32(lm[x] / null[x])))
                m.rmesc[v, x] = f32(sreLOG2(f32(rm[x] / null[x])))
            _fexpect_sc_vec(m.lmesc[v], null)
            _fexpect_sc_vec(m.rmesc[v], null)
            _iexpect_sc_vec(m.ilmesc[v], null)
            _iexpect_sc_vec(m.irmesc[v], null)
        elif st in (ML_st, MR_st, IL_st, IR_st):
            for x in range(K):
                esc[v, x] = f32(sreLOG2(f32(m.e[v, x] / null[x])))
                iesc[v, x] = Prob2Score(m.e[v, x], null[x])
            if st in (ML_st, IL_st):
                m.lmesc[v, :K] = esc[v, :K]
                m.ilmesc[v, :K] = iesc[v, :K]
                m.rmesc[v, :K] = 0.0
                m.irmesc[v, :K] = 0
                _fexpect_sc_vec(m.lmesc[v], null)
                _iexpect_sc_vec(m.ilmesc[v], null)
                m.rmesc[v, K + 1: Kp - 2] = 0.0
                m.irmesc[v, K + 1: Kp - 2] = 0
            else:
                m.lmesc[v, :K] = 0.0
                m.ilmesc[v, :K] = 0
                m.rmesc[v, :K] = esc[v, :K]
                m.irmesc[v, :K] = iesc[v, :K]
                m.lmesc[v, K + 1: Kp - 2] = 0.0
                m.ilmesc[v, K + 1: Kp - 2] = 0
                _fexpect_sc_vec(m.rmesc[v], null)
                _iexpect_sc_vec(m.irmesc[v], null)
        m.beginsc[v] = f32(sreLOG2(m.begin[v]))
        m.ibeginsc[v] = Prob2Score(m.begin[v], 1.0)
        m.endsc[v] = f32(sreLOG2(m.end[v]))
        m.iendsc[v] = Prob2Score(m.end[v], 1.0)
    m.iel_selfsc = Prob2Score(f32(sreEXP2(m.el_selfsc)), 1.0)
    # optimised emission tables (src/cm.c:3604 FCalcOptimizedEmitScores)
    oesc = np.full((M, Kp * Kp), f32(IMPOSSIBLE), np.float32)
    ioesc = np.full((M, Kp * Kp), -INFTY, np.int32)
    left = {a: _fcount(a) for a in range(K + 1, Kp - 1)}
    for v in range(M):
        st = m.sttype[v]
        if st in (IL_st, ML_st, IR_st, MR_st):
            for a in range(K):
                oesc[v, a] = esc[v, a]
                ioesc[v, a] = iesc[v, a]
            oesc[v, K] = f32(IMPOSSIBLE)
            ioesc[v, K] = -INFTY
            for a in range(K + 1, Kp - 1):
                oesc[v, a] = _favg_score(a, esc[v])
                ioesc[v, a] = int(math.floor(0.5 + float(f32(INTSCALE * oesc[v, a]))))
            oesc[v, Kp - 1] = f32(IMPOSSIBLE)
            ioesc[v, Kp - 1] = -INFTY
        elif st == MP_st:
            for a in range(K):
                for b in range(K):
                    oesc[v, a * Kp + b] = esc[v, a * K + b]
                    ioesc[v, a * Kp + b] = iesc[v, a * K + b]
            for a in range(K + 1, Kp - 1):          # left degenerate, right canonical
                for b in range(K):
                    s = f32(0.0)
                    for l in range(K):
                        s = f32(s + f32(esc[v, l * K + b] * left[a][l]))
                    oesc[v, a * Kp + b] = s
            for a in range(K):                       # left canonical, right degenerate
                for b in range(K + 1, Kp - 1):
                    s = f32(0.0)
                    for r in range(K):
                        s = f32(s + f32(esc[v, a * K + r] * left[b][r]))
                    oesc[v, a * Kp + b] = s
            for a in range(K + 1, Kp - 1):          # both degenerate
                for b in range(K + 1, Kp - 1):
                    s = f32(0.0)
                    for l in range(K):
                        for r in range(K):
                            s = f32(s + f32(f32(esc[v, l * K + r] * left[a][l]) * left[b][r]))
                    oesc[v, a * Kp + b] = s
            for a in range(Kp):
                for b in range(Kp):
                    if (a < K and b < K) or a in (K, Kp - 1) or b in (K, Kp - 1):
                        continue
                    ioesc[v, a * Kp + b] = int(math.floor(0.5 + float(f32(INTSCALE * oesc[v, a * Kp + b]))))
    m.oesc, m.ioesc = oesc, ioesc
    m.configured = True
    if m.t_global is not None and m.plast is not None:
        truncation_tables(m)
    return m


def load(path: str, which: int = 0, local: bool = True) -> CMModel:
    """Read and configure a CM for scanning."""
    return truncation_tables(configure(read_cm(path, which), local=local))


# ---- query-dependent bands ---------------------------------------------------
def _dsum_kahan(v) -> float:
    """Easel esl_vec_DSum: compensated double sum."""
    s, c = 0.0, 0.0
    for x in v:
        y = float(x) - c
        t = s + y
        c = (t - s) - y
        s = t
    return s


def qdb_bands(m: CMModel, beta1: float = 1e-7, beta2: float = 1e-15, beta_W: float = 1e-7):
    """Query-dependent bands and W: CalculateQueryDependentBands /
    BandCalculationEngine (src/cm_qdband.c:45-451).

    gamma[v][n] is the probability that the subtree rooted at v emits n
    residues, computed from the leaves up in double precision over the
    transitions before local configuration, with local begins (from pbegin)
    into the root and local ends off.  dmin/dmax cut <= beta of probability
    mass off each tail (beta1 -> dmin1/dmax1, beta2 -> dmin2/dmax2); W is the
    root's right bound at beta_W.  The maximum length Z starts at 4 clen and
    doubles until the truncated tail is negligible.  Every sum runs in the
    reference's order, so the integer bounds agree exactly.
    Returns (dmin1, dmax1, dmin2, dmax2, W) as int32 arrays and an int."""
    if beta2 - beta1 > 1e-20:
        raise ValueError("qdb_bands: beta1 must be >= beta2")
    max_beta = max(beta_W, beta1, beta2)
    M = m.M
    t = m.t_global.astype(np.float64)          # float probabilities, used as doubles
    internal = (MATP_nd, MATL_nd, MATR_nd, BIF_nd)
    nstarts = sum(1 for nd in range(2, m.nodes) if m.ndtype[nd] in internal)
    begin = np.zeros(M, np.float32)
    begin[m.nodemap[1]] = f32(1.0 - float(m.pbegin))
    pb = f32(f32(m.pbegin) / f32(nstarts))
    for nd in range(2, m.nodes):
        if m.ndtype[nd] in internal:
            begin[m.nodemap[nd]] = pb
    Z = m.clen * 4
    while True:
        res = _band_engine(m, Z, t, begin, beta1, beta2, beta_W, max_beta)
        if res is not None:
            return res
        Z *= 2
        if Z > m.clen * 1000:
            raise ValueError("qdb_bands: Z got insanely large (> 1000*clen)")


def _band_engine(m, Z, t, begin, beta1, beta2, beta_W, max_beta):
    """One pass of BandCalculationEngine at maximum length Z; None when the
    truncation error is not negligible (the caller doubles Z)."""
    M = m.M
    eps = np.finfo(np.float64).eps
    gamma = [None] * M
    g0 = np.zeros(Z + 1)
    gE = np.zeros(Z + 1)
    gE[0] = 1.0
    dmin1, dmax1 = np.zeros(M, np.int32), np.zeros(M, np.int32)
    dmin2, dmax2 = np.zeros(M, np.int32), np.zeros(M, np.int32)
    W = 0
    for v in range(M - 1, -1, -1):
        st = int(m.sttype[v])
        if st == E_st:
            gamma[v] = gE
            continue
        if v == 0:
            g = g0
        else:
            g = np.zeros(Z + 1)
            if st == B_st:
                gw, gy = gamma[int(m.cfirst[v])], gamma[int(m.cnum[v])]
                for leftn in range(Z + 1):          # per n, terms added in leftn order
                    g[leftn:] += gw[leftn] * gy[: Z + 1 - leftn]
            else:
                dv = 2 if st == MP_st else (1 if st in (ML_st, MR_st, IL_st, IR_st) else 0)
                ys = [int(m.cfirst[v]) + yo for yo in range(int(m.cnum[v]))]
                if v in ys:
                    # an insert's self-loop reads its own density at n - dv:
                    # sequential in n, children summed in yoffset order
                    tv = [float(t[v, yo]) for yo in range(len(ys))]
                    cols = [None if y == v else gamma[y].tolist() for y in ys]
                    gl = [0.0] * (Z + 1)
                    for n in range(dv, Z + 1):
                        acc = 0.0
                        for yo, y in enumerate(ys):
                            acc += tv[yo] * (gl[n - dv] if y == v else cols[yo][n - dv])
                        gl[n] = acc
                    g[:] = gl
                else:
                    for yo, y in enumerate(ys):
                        g[dv:] += float(t[v, yo]) * gamma[y][: Z + 1 - dv]
            gamma[v] = g
        pdf = float(np.cumsum(g)[-1]) if v != 0 else 0.0
        if begin[v] > 0.0:
            g0 += float(begin[v]) * g
        if v == 0:
            pdf = _dsum_kahan(g0)
        if pdf <= 0.999 or g[Z] > max_beta * eps:
            return None
        if pdf > 1.0:
            s = _dsum_kahan(g)
            g /= s
        c = np.cumsum(g)
        k2 = int(np.argmax(c > beta2))
        k1 = k2 + int(np.argmax(c[k2:] > beta1))
        dmin2[v], dmin1[v] = k2, k1
        r = np.cumsum(g[::-1])
        k2 = int(np.argmax(r > beta2))
        k1 = k2 + int(np.argmax(r[k2:] > beta1))
        dmax2[v], dmax1[v] = Z - k2, Z - k1
        if v == 0:
            W = Z - int(np.argmax(r > beta_W))
    for b in (W, int(dmax1[0]), int(dmax2[0])):
        if not _band_truncation_negligible(g0, b, Z):
            return None
    return dmin1, dmax1, dmin2, dmax2, W


def _band_truncation_negligible(density, b, Z) -> bool:
    """BandTruncationNegligible (src/cm_qdband.c:520-545)."""
    C = 0.0
    for i in range(b + 1, Z + 1):
        C += float(density[i])
    logbeta = (math.log(density[Z]) - math.log(density[b + 1])) / (Z - b - 1)
    beta = math.exp(logbeta)
    D = (beta / (1.0 - beta)) * float(density[Z])
    return D < C * np.finfo(np.float64).eps


# ---- truncated-scan tables ----------------------------------------------------
def emit_map(m: CMModel):
    """Consensus coordinates of every node: CreateEmitMap (src/display.c:1110).
    A depth-first walk of the guide tree counts consensus columns; lpos[nd] is
    the column at the node's left side, rpos[nd] one past its right side.
    Returns (lpos, rpos) as int32 arrays of length ``nodes``."""
    lpos = np.full(m.nodes, -1, np.int32)
    rpos = np.full(m.nodes, -1, np.int32)
    cpos = 0
    stack = [(0, False)]
    while stack:
        nd, on_right = stack.pop()
        t = int(m.ndtype[nd])
        if on_right:
            rpos[nd] = cpos + 1
            if t in (MATP_nd, MATR_nd):
                cpos += 1
            continue
        if t in (MATP_nd, MATL_nd):
            cpos += 1
        lpos[nd] = cpos
        stack.append((nd, True))
        if t == BIF_nd:
            v = int(m.nodemap[nd])
            stack.append((int(m.ndidx[m.cnum[v]]), False))     # right subtree, visited second
            stack.append((int(m.ndidx[m.cfirst[v]]), False))   # left subtree, visited first
        elif t != END_nd:
            stack.append((nd + 1, False))
    if (lpos < 0).any() or (rpos < 0).any():
        raise ValueError("emit map: unreachable node")
    return lpos, rpos


def _detached(m: CMModel, v: int) -> bool:
    """StateIsDetached (src/cm.c:1775): the state just before an END_E."""
    return v + 1 < m.M and int(m.stid[v + 1]) == END_E


def state_occupancy(m: CMModel) -> np.ndarray:
    """Expected number of visits of each state in a global parse,
    cm_ExpectedStateOccupancy (src/cm.c:4250-4330), over the transitions
    before local configuration.  A parent x reaches child v through its
    transition v - cfirst[x]; an insert adds its self-loop's geometric
    series.  Double precision, as the reference."""
    t = m.t_global
    psi = np.zeros(m.M, np.float64)
    for v in range(m.M):
        st = int(m.sttype[v])
        if st == S_st:
            psi[v] = 1.0
            continue
        ins = st in (IL_st, IR_st)
        acc = 0.0
        for y in range(int(m.pnum[v]) - 1, (1 if ins else 0) - 1, -1):
            x = int(m.plast[v]) - y
            acc += psi[x] * float(t[x, v - int(m.cfirst[x])])
        if ins:
            acc += acc * (float(t[v, 0]) / (1.0 - float(t[v, 0])))
        psi[v] = acc
    return psi


def _inserts_of_node(m: CMModel, nd: int):
    """InsertsGivenNodeIndex (src/cm.c:4897): insert states of node nd."""
    v = int(m.nodemap[nd])
    t = int(m.ndtype[nd])
    if t == MATP_nd:
        return v + 4, v + 5
    if t in (MATL_nd, MATR_nd):
        return v + 2, -1
    if t == BEGR_nd:
        return v + 1, -1
    if t == ROOT_nd:
        return v + 1, v + 2
    return -1, -1


def truncation_tables(m: CMModel) -> CMModel:
    """Truncated-begin penalties and emit map of a CM: cm_tr_penalties_Create
    (src/cm_trunc.c:51-440) with cm_CalculateLocalBeginProbs
    (src/cm_modelconfig.c:397) and CreateEmitMap (src/display.c:1110).

    Fills m.emap_lpos/emap_rpos and the [3, M] tables tr_g_pty, tr_l_pty
    (float, log2 probabilities, IMPOSSIBLE where no truncated begin is
    allowed) and tr_ig_pty, tr_il_pty (integer scores, -INFTY), indexed
    [pty_idx][v] with pty_idx 0 = 5' and 3', 1 = 5' only, 2 = 3' only.
    The penalties are probabilities until the final conversion; states the
    conversion skips (detached inserts) keep their probability in the float
    tables, as the reference does."""
    if getattr(m, "tr_g_pty", None) is not None:
        return m
    M = m.M
    lpos_map, rpos_map = emit_map(m)
    m.emap_lpos, m.emap_rpos = lpos_map, rpos_map
    psi = state_occupancy(m)
    # local begin probabilities from pbegin (cm_CalculateLocalBeginProbs)
    internal = (MATP_nd, MATL_nd, MATR_nd, BIF_nd)
    nstarts = sum(1 for nd in range(2, m.nodes) if m.ndtype[nd] in internal)
    begin = np.zeros(M, np.float32)
    begin[m.nodemap[1]] = f32(1.0 - float(m.pbegin))
    pb = f32(f32(m.pbegin) / f32(nstarts))
    for nd in range(2, m.nodes):
        if m.ndtype[nd] in internal:
            begin[m.nodemap[nd]] = pb
    P53, P5, P3 = 0, 1, 2
    g = np.full((3, M), f32(IMPOSSIBLE), np.float32)
    l = np.full((3, M), f32(IMPOSSIBLE), np.float32)
    g_5and3 = f32(2.0 / (m.clen * (m.clen + 1)))
    g_5or3 = f32(1.0 / m.clen)
    prv5 = prv3 = prv53 = f32(0.0)
    for nd in range(m.nodes):
        t = int(m.ndtype[nd])
        lpos = int(lpos_map[nd]) if t in (MATP_nd, MATL_nd) else int(lpos_map[nd]) + 1
        rpos = int(rpos_map[nd]) if t in (MATP_nd, MATR_nd) else int(rpos_map[nd]) - 1
        if t == END_nd:
            prv5 = prv3 = prv53 = f32(0.0)
        elif t in (BEGL_nd, BEGR_nd):
            b = int(m.plast[m.nodemap[nd]])          # the parent bifurcation
            prv5 = f32(0.0) if t == BEGL_nd else l[P5, b]
            prv3 = f32(0.0) if t == BEGR_nd else l[P3, b]
            prv53 = l[P53, b]
        elif t in internal:
            s = int(m.nodemap[nd])
            i1, i2 = _inserts_of_node(m, nd - 1)
            # (the reference's extra MATP pair-state term compares a node type
            # with a state id and never applies, so m_psi is psi[s] alone)
            m_psi = f32(psi[s])
            i1_psi = f32(psi[i1]) if i1 != -1 else f32(0.0)
            i2_psi = f32(psi[i2]) if i2 != -1 else f32(0.0)
            summed = f32(f32(m_psi + i1_psi) + i2_psi)
            shares = [(s, f32(m_psi / summed))]
            if i1 != -1:
                shares.append((i1, f32(i1_psi / summed)))
            if i2 != -1:
                shares.append((i2, f32(i2_psi / summed)))
            for x, w in shares:
                if g[P53, x] > -9.999e35 or l[P53, x] > -9.999e35:
                    raise ValueError(f"truncation penalty of state {x} set twice")
                g[P53, x] = f32(w * g_5and3)
                if rpos == m.clen:
                    g[P5, x] = f32(w * g_5or3)
                if lpos == 1:
                    g[P3, x] = f32(w * g_5or3)
            sub = rpos - lpos + 1
            nfrag53 = (sub * (sub + 1)) // 2
            cur5 = f32(f32(begin[s] / f32(sub)) + prv5)
            cur3 = f32(f32(begin[s] / f32(sub)) + prv3)
            cur53 = f32(f32(begin[s] / f32(nfrag53)) + prv53)
            for x, w in shares:
                l[P53, x] = f32(w * cur53)
                l[P5, x] = f32(w * cur5)
                l[P3, x] = f32(w * cur3)
            prv5 = cur5 if t == MATL_nd else f32(0.0)
            prv3 = cur3 if t == MATR_nd else f32(0.0)
            prv53 = cur53
    ig = np.full((3, M), -INFTY, np.int32)
    il = np.full((3, M), -INFTY, np.int32)
    for v in range(M):
        sid, st = int(m.stid[v]), int(m.sttype[v])
        if not (sid in (MATP_MP, MATL_ML, MATR_MR, BIF_B) or (st in (IL_st, IR_st) and not _detached(m, v))):
            continue
        if sid == MATP_IL and int(m.ndtype[int(m.ndidx[v]) + 1]) == END_nd:
            continue
        if not g[P53, v] > -9.999e35:
            raise ValueError(f"state {v}: missing global truncation penalty")
        for p in (P53, P5, P3):
            if g[p, v] > -9.999e35:
                ig[p, v] = Prob2Score(g[p, v], 1.0)
                g[p, v] = f32(sreLOG2(g[p, v]))
            if not l[p, v] > -9.999e35:
                raise ValueError(f"state {v}: missing local truncation penalty")
            il[p, v] = Prob2Score(l[p, v], 1.0)
            l[p, v] = f32(sreLOG2(l[p, v]))
    m.tr_g_pty, m.tr_l_pty, m.tr_ig_pty, m.tr_il_pty = g, l, ig, il
    return m


# ---- ctypes view of cmgb_model_desc -----------------------------------------
_p = ctypes.c_void_p


class ModelDesc(ctypes.Structure):
    """Mirror of cmgb_model_desc (include/infernal_gb300.h)."""
    _fields_ = [("M", ctypes.c_int), ("W", ctypes.c_int), ("K", ctypes.c_int), ("Kp", ctypes.c_int),
                ("flags", ctypes.c_int),
                ("sttype", _p), ("stid", _p), ("cfirst", _p), ("cnum", _p),
                ("dmin1", _p), ("dmax1", _p), ("dmin2", _p), ("dmax2", _p),
                ("tsc", _p), ("oesc", _p), ("endsc", _p), ("beginsc", _p), ("el_selfsc", ctypes.c_float),
                ("itsc", _p), ("ioesc", _p), ("iendsc", _p), ("ibeginsc", _p), ("iel_selfsc", ctypes.c_int),
                ("null", _p), ("null3_omega", ctypes.c_float),
                ("lmesc", _p), ("rmesc", _p), ("ilmesc", _p), ("irmesc", _p),
                ("tr_g_pty", _p), ("tr_l_pty", _p), ("tr_ig_pty", _p), ("tr_il_pty", _p),
                ("ndidx", _p), ("emap_lpos", _p), ("emap_rpos", _p), ("clen", ctypes.c_int),
                ("ndtype", _p), ("nodes", ctypes.c_int)]


def make_desc(m: CMModel, flags_extra: int = 0, keep: Optional[list] = None) -> ModelDesc:
    """Builds a ModelDesc pointing into contiguous copies of m's arrays.
    The copies are appended to ``keep`` (which the caller must hold)."""
    keep = [] if keep is None else keep

    def ptr(a, dt):
        if a is None:
            return None
        c = np.ascontiguousarray(a, dtype=dt)
        keep.append(c)
        return c.ctypes.data

    d = ModelDesc()
    d.M, d.W, d.K, d.Kp = m.M, m.W, m.K, m.Kp
    d.flags = int(m.flags | flags_extra)
    d.sttype, d.stid = ptr(m.sttype, np.int8), ptr(m.stid, np.int8)
    d.cfirst, d.cnum = ptr(m.cfirst, np.int32), ptr(m.cnum, np.int32)
    d.dmin1, d.dmax1 = ptr(m.dmin1, np.int32), ptr(m.dmax1, np.int32)
    d.dmin2, d.dmax2 = ptr(m.dmin2, np.int32), ptr(m.dmax2, np.int32)
    d.tsc, d.oesc = ptr(m.tsc, np.float32), ptr(m.oesc, np.float32)
    d.endsc, d.beginsc = ptr(m.endsc, np.float32), ptr(m.beginsc, np.float32)
    d.el_selfsc = float(m.el_selfsc)
    d.itsc, d.ioesc = ptr(m.itsc, np.int32), ptr(m.ioesc, np.int32)
    d.iendsc, d.ibeginsc = ptr(m.iendsc, np.int32), ptr(m.ibeginsc, np.int32)
    d.iel_selfsc = int(m.iel_selfsc)
    d.null, d.null3_omega = ptr(m.null, np.float32), float(m.null3_omega)
    d.lmesc, d.rmesc = ptr(m.lmesc, np.float32), ptr(m.rmesc, np.float32)
    d.ilmesc, d.irmesc = ptr(m.ilmesc, np.int32), ptr(m.irmesc, np.int32)
    d.ndidx = ptr(m.ndidx, np.int32)
    d.clen = m.clen
    if getattr(m, "tr_g_pty", None) is not None:
        d.tr_g_pty, d.tr_l_pty = ptr(m.tr_g_pty, np.float32), ptr(m.tr_l_pty, np.float32)
        d.tr_ig_pty, d.tr_il_pty = ptr(m.tr_ig_pty, np.int32), ptr(m.tr_il_pty, np.int32)
        d.emap_lpos, d.emap_rpos = ptr(m.emap_lpos, np.int32), ptr(m.emap_rpos, np.int32)
    d.ndtype = ptr(m.ndtype, np.int8)
    d.nodes = m.nodes
    d._keep = keep
    return d


# ---- flat (npz) serialisation of a configured model --------------------------
_ARRAYS = ("sttype", "stid", "ndidx", "cfirst", "cnum", "plast", "pnum", "ndtype", "nodemap",
           "dmin1", "dmax1", "dmin2", "dmax2", "null", "tsc", "itsc", "oesc", "ioesc",
           "endsc", "beginsc", "iendsc", "ibeginsc", "lmesc", "rmesc", "ilmesc", "irmesc", "t_global", "e")
_SCALARS = ("M", "nodes", "clen", "W", "K", "Kp", "flags", "iel_selfsc")
_F32 = ("el_selfsc", "null3_omega", "pbegin", "pend")


def save_npz(m: CMModel, path: str) -> None:
    """Writes the configured score tables of m to a compressed .npz."""
    d = {a: getattr(m, a) for a in _ARRAYS}
    for s in _SCALARS:
        d[s] = np.int64(getattr(m, s))
    for s in _F32:
        d[s] = np.float32(getattr(m, s))
    d["name"] = np.array(m.name)
    for tag, vals in (m.ecm or {}).items():     # E-value calibration lines (ECMLC, ECMGC, ECMLI, ECMGI)
        d["ecm_" + tag] = np.array(vals, np.float64)
    np.savez_compressed(path, **d)


def load_npz(path: str) -> CMModel:
    """Reads a model written by save_npz."""
    z = np.load(path)
    m = CMModel(name=str(z["name"]), M=int(z["M"]), nodes=int(z["nodes"]), clen=int(z["clen"]),
                W=int(z["W"]))
    for a in _ARRAYS:
        setattr(m, a, z[a] if a in z else None)
    for s in _SCALARS:
        setattr(m, s, int(z[s]))
    for s in _F32:
        setattr(m, s, f32(z[s]))
    m.configured = True
    m.ecm = {k[4:]: tuple(float(x) for x in z[k]) for k in z.files if k.startswith("ecm_")}
    if m.t_global is not None and m.plast is not None:
        truncation_tables(m)
    return m
