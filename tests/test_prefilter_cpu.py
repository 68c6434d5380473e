"""CPU tests of the pre-filter's training-data helpers (no GPU): the
doublet-preserving shuffle, the fast CM sampler against the reference-style
walk, the bulk window block and the operating-point table."""
import random
from collections import Counter

import numpy as np

from infernal_gb300 import cmfile, emit, prefilter


def _dinucs(s):
    return Counter(s[i:i + 2] for i in range(len(s) - 1))


def test_dinuc_shuffle_preserves_doublets_and_ends():
    rng = np.random.default_rng(3)
    for n in (3, 17, 400):
        s = "".join(rng.choice(list("ACGU"), n))
        t = prefilter.dinuc_shuffle(s, rng)
        assert len(t) == n and t[0] == s[0] and t[-1] == s[-1]
        assert _dinucs(t) == _dinucs(s)


def test_fast_sampler_matches_the_walk_in_distribution(models):
    """emit.Sampler draws from the same model as emit.sample (a different
    random stream): mean length and composition agree within sampling error;
    a seed gives the same sequence every time."""
    m = models["Vault"]
    S = emit.Sampler(m)
    a = [S.sample(random.Random(k)) for k in range(400)]
    assert S.sample(random.Random(7)) == a[7]
    rng = np.random.default_rng(1)
    b = [emit.sample(m, rng) for _ in range(400)]
    la, lb = np.array([len(x) for x in a]), np.array([len(x) for x in b])
    assert abs(la.mean() - lb.mean()) < 4 * np.sqrt(la.var() / 400 + lb.var() / 400) + 1e-9
    ca, cb = Counter("".join(a)), Counter("".join(b))
    for x in "ACGU":
        assert abs(ca[x] / sum(ca.values()) - cb[x] / sum(cb.values())) < 0.02


def test_window_block_layout(models):
    m = models["tRNA"]
    blk = prefilter.make_window_block(m, 90, seed=5)
    W2 = 2 * m.W
    assert blk.shape == (90, W2 + 2) and blk.dtype == np.uint8
    assert (blk[:, 0] == cmfile.DSQ_SENTINEL).all() and (blk[:, -1] == cmfile.DSQ_SENTINEL).all()
    assert blk[:, 1:-1].max() <= 3
    assert np.array_equal(blk, prefilter.make_window_block(m, 90, seed=5))      # seeded


def test_operating_points_table():
    rng = np.random.default_rng(0)
    n = 3000
    best = np.full(n, -np.inf, np.float32)
    best[:600] = rng.uniform(15, 40, 600)                  # windows with a final hit
    logit = np.where(np.isfinite(best), rng.normal(2, 1, n), rng.normal(-2, 1, n)).astype(np.float32)
    bg = np.arange(n) >= 2000
    pts = prefilter.operating_points(logit, best, bg, bits=(15.0, 25.0), recalls=(0.9, 0.99))
    assert pts.shape == (4, 5)
    for b in (15.0, 25.0):
        rows = pts[pts[:, 0] == b]
        for q, t in rows[:, 1:3]:
            assert (logit[best >= b] > t).mean() >= q
        assert rows[1, 2] <= rows[0, 2]                     # higher recall, lower threshold
        assert rows[1, 3] >= rows[0, 3]                     # ... and more negatives kept


def test_window_block_multi_layout(models):
    """Windows for a several-head filter: 2 Wmax residues, the kinds cycle
    through every model's emitted windows, background and shuffles."""
    ms = [models["tRNA"], models["Vault"]]
    blk, src = prefilter.make_window_block_multi(ms, 40, seed=3)
    W2 = 2 * max(m.W for m in ms)
    assert blk.shape == (40, W2 + 2)
    assert (blk[:, 0] == cmfile.DSQ_SENTINEL).all() and blk[:, 1:-1].max() <= 3
    kinds = np.arange(40) % 4
    assert (src[kinds == 0] == 0).all() and (src[kinds == 1] == 1).all()
    assert (src[kinds == 2] == -1).all() and (src[kinds == 3] == -2).all()
    blk2, src2 = prefilter.make_window_block_multi(ms, 40, seed=3)
    assert np.array_equal(blk, blk2) and np.array_equal(src, src2)
