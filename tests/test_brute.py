"""Exhaustive check on hand-specified tiny CMs, after the reference's
"brute" integration test (src/itest_brute.c): hand-specified models with
random parameters -- four nodes (ROOT, MATL, MATL, END; ten states), and
eight nodes with a bifurcation and a base pair (ROOT, BIF, BEGL, MATP, END,
BEGR, MATL, END; eighteen states) -- configured in global mode and in local
mode (local begins into the internal nodes, local ends through EL).
Every parse of every subsequence of short random targets is scored by a
top-down recursion written from the model's definition -- the maximum over
parses (CYK) in float32 with the scanners' two-term additions, the sum over
parses (Inside) in exact double log-space, except that an empty subsequence
at an S or D state takes the maximum of its alternatives, which is how the
reference's matrix initialisation defines those cells -- and the best root
score over all subsequences is compared with the scanners' best score: CYK exactly,
integer and float Inside within the log-sum tables' error.  The oracle and
the emulated kernel run on the CPU, the kernels on the GPU."""
import functools
import math

import numpy as np
import pytest

import oracle
from infernal_gb300 import cmfile, lib as L

D, MP, ML, MR, IL, IR, S, E, B = (cmfile.D_st, cmfile.MP_st, cmfile.ML_st, cmfile.MR_st, cmfile.IL_st, cmfile.IR_st,
                                  cmfile.S_st, cmfile.E_st, cmfile.B_st)
IMP = float(np.float32(cmfile.IMPOSSIBLE))
ND = cmfile

# Topologies: per state (type, unique id, node index, cfirst, cnum); children
# of a state are cfirst .. cfirst + cnum - 1 (inserts list themselves first);
# a B state's cfirst is its BEGL_S and its cnum its BEGR_S.
TOPOLOGIES = {
    # ROOT (S IL IR), MATL (ML D IL), MATL (ML D IL), END (E)
    "matl": dict(
        states=[(S, 0, 0, 1, 4), (IL, 1, 0, 1, 4), (IR, 2, 0, 2, 3),
                (ML, 12, 1, 5, 3), (D, 13, 1, 5, 3), (IL, 14, 1, 5, 3),
                (ML, 12, 2, 8, 2), (D, 13, 2, 8, 2), (IL, 14, 2, 8, 2),
                (E, 18, 3, -1, 0)],
        nodes=[ND.ROOT_nd, ND.MATL_nd, ND.MATL_nd, ND.END_nd], clen=2),
    # ROOT (S IL IR), BIF (B), BEGL (S), MATP (MP ML MR D IL IR), END (E),
    # BEGR (S IL), MATL (ML D IL), END (E)
    "bif": dict(
        states=[(S, 0, 0, 1, 3), (IL, 1, 0, 1, 3), (IR, 2, 0, 2, 2),
                (B, 19, 1, 4, 12),
                (S, 3, 2, 5, 4),
                (MP, 6, 3, 9, 3), (ML, 7, 3, 9, 3), (MR, 8, 3, 9, 3), (D, 9, 3, 9, 3), (IL, 10, 3, 9, 3), (IR, 11, 3, 10, 2),
                (E, 18, 4, -1, 0),
                (S, 4, 5, 13, 3), (IL, 5, 5, 13, 3),
                (ML, 12, 6, 16, 2), (D, 13, 6, 16, 2), (IL, 14, 6, 16, 2),
                (E, 18, 7, -1, 0)],
        nodes=[ND.ROOT_nd, ND.BIF_nd, ND.BEGL_nd, ND.MATP_nd, ND.END_nd, ND.BEGR_nd, ND.MATL_nd, ND.END_nd], clen=3),
}


def tiny_cm(rng, W=10, local=False, topology="matl"):
    T = TOPOLOGIES[topology]
    st = T["states"]
    M, nodes = len(st), len(T["nodes"])
    m = cmfile.CMModel(name="brute", M=M, nodes=nodes, clen=T["clen"], W=W)
    m.sttype = np.array([x[0] for x in st], np.int8)
    m.stid = np.array([x[1] for x in st], np.int8)
    m.ndidx = np.array([x[2] for x in st], np.int32)
    m.cfirst = np.array([x[3] for x in st], np.int32)
    m.cnum = np.array([x[4] for x in st], np.int32)
    m.ndtype = np.array(T["nodes"], np.int8)
    m.nodemap = np.array([min(v for v in range(M) if st[v][2] == nd) for nd in range(nodes)], np.int32)
    m.t = np.zeros((M, 6), np.float32)
    m.e = np.zeros((M, 16), np.float32)
    for v, (t, _, _, _, cn) in enumerate(st):
        if t not in (B, E) and cn:
            m.t[v, :cn] = rng.dirichlet(np.ones(cn))
        if t == MP:
            m.e[v, :16] = rng.dirichlet(np.ones(16))
        elif t in (ML, MR, IL, IR):
            m.e[v, :4] = rng.dirichlet(np.ones(4))
    m.null = np.full(4, 0.25, np.float32)
    m.null3_omega = np.float32(2.0 ** -16)
    m.dmin1 = m.dmax1 = m.dmin2 = m.dmax2 = None
    m.el_selfsc = np.float32(math.log2(0.94))       # EL self-loop (local ends emit through EL)
    return cmfile.configure(m, local=local)


def brute(m, x):
    """Best root score over all subsequences x[i..j] (1-based, j >= i):
    (CYK max over parses in float32, Inside log2-sum over parses in double).
    Local mode: a state with a local end may leave for EL, which emits the
    rest of its subsequence at el_selfsc per residue (after the state's own
    emission); a parse may start at any state with a local begin (the best
    begin is taken by max, also for Inside, as the scanners do)."""
    f32 = np.float32
    tsc, esc = m.tsc, m.oesc
    el, endsc, beginsc = f32(m.el_selfsc), m.endsc, m.beginsc
    STTYPE, CFIRST, CNUM, Kp = [int(t) for t in m.sttype], [int(c) for c in m.cfirst], [int(c) for c in m.cnum], m.Kp

    def shape(v, i, j):
        """(child i, child j, emission score or None); None when v cannot emit here."""
        t = STTYPE[v]
        if t in (ML, IL):
            return (i + 1, j, esc[v, x[i - 1]]) if i <= j else None
        if t in (MR, IR):
            return (i, j - 1, esc[v, x[j - 1]]) if i <= j else None
        if t == MP:
            return (i + 1, j - 1, esc[v, x[i - 1] * Kp + x[j - 1]]) if i < j else None
        return (i, j, None)

    @functools.lru_cache(maxsize=None)
    def cyk(v, i, j):          # parse of x[i..j] (empty when i > j) rooted at state v
        t = STTYPE[v]
        if t == E:
            return f32(0.0) if i > j else f32(IMP)
        if t == B:             # split into BEGL x[i..k] and BEGR x[k+1..j], either part may be empty
            best = f32(IMP)
            for k in range(i - 1, j + 1):
                a, b = cyk(CFIRST[v], i, k), cyk(CNUM[v], k + 1, j)
                if a > IMP / 2 and b > IMP / 2:
                    s = f32(a + b)
                    best = s if s > best else best
            return best
        sh = shape(v, i, j)
        if sh is None:
            return f32(IMP)
        ci, cj, e = sh
        best = f32(IMP)
        for o in range(CNUM[v]):
            c = cyk(CFIRST[v] + o, ci, cj)
            if c > IMP / 2:
                s = f32(c + tsc[v, o])
                best = s if s > best else best
        if endsc[v] > IMP / 2:                       # local end: EL emits the remaining residues
            s = f32(f32(el * f32(max(0, cj - ci + 1))) + endsc[v])
            best = s if s > best else best
        if best <= IMP / 2:
            return f32(IMP)
        return f32(best + e) if e is not None else best

    def lsum(terms):
        terms = [a for a in terms if a > IMP / 2]
        if not terms:
            return -math.inf
        mx = max(terms)
        return mx + math.log2(sum(2.0 ** (a - mx) for a in terms))

    @functools.lru_cache(maxsize=None)
    def ins(v, i, j):          # log2 of the summed probability-odds of all parses
        t = STTYPE[v]
        if t == E:
            return 0.0 if i > j else -math.inf
        if t == B:
            return lsum([ins(CFIRST[v], i, k) + ins(CNUM[v], k + 1, j) for k in range(i - 1, j + 1)])
        sh = shape(v, i, j)
        if sh is None:
            return -math.inf
        ci, cj, e = sh
        e = 0.0 if e is None else float(e)
        terms = [ins(CFIRST[v] + o, ci, cj) + float(tsc[v, o]) for o in range(CNUM[v])]
        if endsc[v] > IMP / 2:
            terms.append(float(el) * max(0, cj - ci + 1) + float(endsc[v]))
        terms = [a for a in terms if a > IMP / 2]
        if not terms:
            return -math.inf
        mx = max(terms)
        if i > j and t in (S, D):
            # empty subsequence: the reference initialises these cells with the
            # MAX over the local end and the children, for Inside too
            # (cm_scan_mx_InitializeIntegers / InitializeFloats, src/cm_mx.c:6039-6138)
            return mx + e
        return mx + math.log2(sum(2.0 ** (a - mx) for a in terms)) + e

    begins = [v for v in range(1, len(STTYPE)) if beginsc[v] > IMP / 2]

    def root_c(i, j):
        b = cyk(0, i, j)
        for v in begins:
            c = cyk(v, i, j)
            if c > IMP / 2:
                s = f32(c + beginsc[v])
                b = s if s > b else b
        return b

    def root_i(i, j):
        return max([ins(0, i, j)] + [ins(v, i, j) + float(beginsc[v]) for v in begins])

    n = len(x)
    best_c = max(root_c(i, j) for j in range(1, n + 1) for i in range(1, j + 1))
    best_i = max(root_i(i, j) for j in range(1, n + 1) for i in range(1, j + 1))
    return float(best_c), best_i


def _cases(n_models=12, local=False, topology="matl"):
    rng = np.random.default_rng([181, int(local), len(topology)])
    for k in range(n_models):
        m = tiny_cm(rng, local=local, topology=topology)
        x = [int(a) for a in rng.integers(0, 4, int(rng.integers(3, 9)))]
        yield k, m, x


def _dsq(x):
    return np.array([cmfile.DSQ_SENTINEL] + x + [cmfile.DSQ_SENTINEL], np.uint8)


@pytest.mark.parametrize("topology,local", [("matl", False), ("matl", True), ("bif", False), ("bif", True)])
def test_brute_oracle(topology, local):
    for k, m, x in _cases(local=local, topology=topology):
        bc, bi = brute(m, x)
        d = _dsq(x)
        c = oracle.scan(m, d, 1, len(x), algo="cyk", qdbidx=0, cutoff=1e30, env_cutoff=1e30)[3]
        i = oracle.scan(m, d, 1, len(x), algo="inside", qdbidx=0, cutoff=1e30, env_cutoff=1e30)[3]
        f = oracle.scan(m, d, 1, len(x), algo="finside", qdbidx=0, cutoff=1e30, env_cutoff=1e30)[3]
        assert np.float32(c) == np.float32(bc), (k, c, bc)
        assert abs(i - bi) < 0.02 and abs(f - bi) < 0.01, (k, i, f, bi)


@pytest.mark.parametrize("topology,local", [("matl", False), ("matl", True), ("bif", False), ("bif", True)])
def test_brute_emulated_kernel(emu, topology, local):
    for k, m, x in list(_cases(local=local, topology=topology))[:4]:
        bc, bi = brute(m, x)
        d = _dsq(x)
        c = emu.scan(m, d, 1, len(x), algo="cyk", qdbidx=0, cutoff=1e30, env_cutoff=1e30).sc
        i = emu.scan(m, d, 1, len(x), algo="inside", qdbidx=0, cutoff=1e30, env_cutoff=1e30).sc
        assert np.float32(c) == np.float32(bc), (k, c, bc)
        assert abs(i - bi) < 0.02, (k, i, bi)


@pytest.mark.gpu
@pytest.mark.parametrize("topology,local", [("matl", False), ("matl", True), ("bif", False), ("bif", True)])
def test_brute_gpu(topology, local):
    s = L.Scanner(0)
    try:
        for k, m, x in _cases(local=local, topology=topology):
            bc, bi = brute(m, x)
            d = _dsq(x)
            c = s.scan(m, d, 1, len(x), algo="cyk", qdbidx=0, cutoff=1e30, env_cutoff=1e30).sc
            i = s.scan(m, d, 1, len(x), algo="inside", qdbidx=0, cutoff=1e30, env_cutoff=1e30).sc
            f = s.scan(m, d, 1, len(x), algo="finside", qdbidx=0, cutoff=1e30, env_cutoff=1e30).sc
            assert np.float32(c) == np.float32(bc), (k, c, bc)
            assert abs(i - bi) < 0.02 and abs(f - bi) < 0.01, (k, i, f, bi)
    finally:
        s.close()


def test_model_without_bands_scans_qdb0_only(emu):
    """A description without band arrays is accepted (qdbidx 0); asking for a
    band set it lacks is an EINCOMPAT error, not a crash."""
    m = tiny_cm(np.random.default_rng(3))
    d = _dsq([0, 1, 2, 3, 0])
    emu.scan(m, d, 1, 5, algo="cyk", qdbidx=0, cutoff=1e30)
    with pytest.raises(L.ScanError) as e:
        emu.scan(m, d, 1, 5, algo="cyk", qdbidx=1, cutoff=1e30)
    assert "band set 1" in str(e.value)
