"""Exhaustive check on hand-specified tiny CMs, after the reference's
"brute" integration test (src/itest_brute.c): a four-node model (ROOT, MATL,
MATL, END; ten states) with random parameters, configured in global mode and in local mode (local
begins into the MATL nodes, a local end through EL).
Every parse of every subsequence of short random targets is scored by a
top-down recursion written from the model's definition -- the maximum over
parses (CYK) in float32 with the scanners' two-term additions, the sum over
parses (Inside) in exact double log-space -- and the best root score over
all subsequences is compared with the scanners' best score: CYK exactly,
integer and float Inside within the log-sum tables' error.  The oracle and
the emulated kernel run on the CPU, the kernels on the GPU."""
import functools
import math

import numpy as np
import pytest

import oracle
from infernal_gb300 import cmfile, lib as L

D, ML, IL, IR, S, E = cmfile.D_st, cmfile.ML_st, cmfile.IL_st, cmfile.IR_st, cmfile.S_st, cmfile.E_st
IMP = float(np.float32(cmfile.IMPOSSIBLE))

# states: ROOT (S IL IR), MATL (ML D IL), MATL (ML D IL), END (E); children of
# a state are cfirst .. cfirst + cnum - 1 (inserts list themselves first)
STTYPE = [S, IL, IR, ML, D, IL, ML, D, IL, E]
STID = [0, 1, 2, 12, 13, 14, 12, 13, 14, 18]      # ROOT_S ROOT_IL ROOT_IR MATL_ML MATL_D MATL_IL ... END_E
CFIRST = [1, 1, 2, 5, 5, 5, 8, 8, 8, -1]
CNUM = [4, 4, 3, 3, 3, 3, 2, 2, 2, 0]


def tiny_cm(rng, W=10, local=False):
    m = cmfile.CMModel(name="brute", M=10, nodes=4, clen=2, W=W)
    m.sttype = np.array(STTYPE, np.int8)
    m.stid = np.array(STID, np.int8)
    m.cfirst = np.array(CFIRST, np.int32)
    m.cnum = np.array(CNUM, np.int32)
    m.ndidx = np.array([0, 0, 0, 1, 1, 1, 2, 2, 2, 3], np.int32)
    m.ndtype = np.array([cmfile.ROOT_nd, cmfile.MATL_nd, cmfile.MATL_nd, cmfile.END_nd], np.int8)
    m.nodemap = np.array([0, 3, 6, 9], np.int32)
    m.t = np.zeros((10, 6), np.float32)
    m.e = np.zeros((10, 16), np.float32)
    for v in range(10):
        if CNUM[v]:
            m.t[v, :CNUM[v]] = rng.dirichlet(np.ones(CNUM[v]))
        if STTYPE[v] in (ML, IL, IR):
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

    @functools.lru_cache(maxsize=None)
    def cyk(v, i, j):          # parse of x[i..j] (empty when i > j) rooted at state v
        t = STTYPE[v]
        if t == E:
            return f32(0.0) if i > j else f32(IMP)
        if t in (ML, IL):
            if i > j:
                return f32(IMP)
            ci, cj, e = i + 1, j, esc[v, x[i - 1]]
        elif t == IR:
            if i > j:
                return f32(IMP)
            ci, cj, e = i, j - 1, esc[v, x[j - 1]]
        else:
            ci, cj, e = i, j, None
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

    @functools.lru_cache(maxsize=None)
    def ins(v, i, j):          # log2 of the summed probability-odds of all parses
        t = STTYPE[v]
        if t == E:
            return 0.0 if i > j else -math.inf
        if t in (ML, IL):
            if i > j:
                return -math.inf
            ci, cj, e = i + 1, j, float(esc[v, x[i - 1]])
        elif t == IR:
            if i > j:
                return -math.inf
            ci, cj, e = i, j - 1, float(esc[v, x[j - 1]])
        else:
            ci, cj, e = i, j, 0.0
        terms = [ins(CFIRST[v] + o, ci, cj) + float(tsc[v, o]) for o in range(CNUM[v])]
        if endsc[v] > IMP / 2:
            terms.append(float(el) * max(0, cj - ci + 1) + float(endsc[v]))
        terms = [a for a in terms if a > IMP / 2]
        if not terms:
            return -math.inf
        mx = max(terms)
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


def _cases(n_models=12, local=False):
    rng = np.random.default_rng(181 + int(local))
    for k in range(n_models):
        m = tiny_cm(rng, local=local)
        x = [int(a) for a in rng.integers(0, 4, int(rng.integers(3, 9)))]
        yield k, m, x


def _dsq(x):
    return np.array([cmfile.DSQ_SENTINEL] + x + [cmfile.DSQ_SENTINEL], np.uint8)


@pytest.mark.parametrize("local", [False, True])
def test_brute_oracle(local):
    for k, m, x in _cases(local=local):
        bc, bi = brute(m, x)
        d = _dsq(x)
        c = oracle.scan(m, d, 1, len(x), algo="cyk", qdbidx=0, cutoff=1e30, env_cutoff=1e30)[3]
        i = oracle.scan(m, d, 1, len(x), algo="inside", qdbidx=0, cutoff=1e30, env_cutoff=1e30)[3]
        f = oracle.scan(m, d, 1, len(x), algo="finside", qdbidx=0, cutoff=1e30, env_cutoff=1e30)[3]
        assert np.float32(c) == np.float32(bc), (k, c, bc)
        assert abs(i - bi) < 0.02 and abs(f - bi) < 0.01, (k, i, f, bi)


@pytest.mark.parametrize("local", [False, True])
def test_brute_emulated_kernel(emu, local):
    for k, m, x in list(_cases(local=local))[:4]:
        bc, bi = brute(m, x)
        d = _dsq(x)
        c = emu.scan(m, d, 1, len(x), algo="cyk", qdbidx=0, cutoff=1e30, env_cutoff=1e30).sc
        i = emu.scan(m, d, 1, len(x), algo="inside", qdbidx=0, cutoff=1e30, env_cutoff=1e30).sc
        assert np.float32(c) == np.float32(bc), (k, c, bc)
        assert abs(i - bi) < 0.02, (k, i, bi)


@pytest.mark.gpu
@pytest.mark.parametrize("local", [False, True])
def test_brute_gpu(local):
    s = L.Scanner(0)
    try:
        for k, m, x in _cases(local=local):
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
