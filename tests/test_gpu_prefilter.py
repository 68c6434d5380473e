"""The learned pre-filter's hand-written BF16 tensor-core kernels
(csrc/filter.cu) against the same network in PyTorch FP32 with the kernel's
BF16 rounding points.  Tolerance: logits within 0.05 + 2% (the two differ
only in FP32 summation order before each BF16 rounding)."""
import numpy as np
import pytest

from infernal_gb300 import cmfile, lib as L, prefilter

pytestmark = pytest.mark.gpu


def _random_weights(rng):
    s = 1.0 / np.sqrt(9 * 128)
    import torch
    w = (rng.standard_normal((5, 9, 128, 128)) * s).astype(np.float32)
    wb = torch.from_numpy(w).to(torch.bfloat16).view(torch.int16).numpy().view(np.uint16)
    return {"w0": (rng.standard_normal((9, 4, 128)) * 0.3).astype(np.float32), "w": wb,
            "bias": (rng.standard_normal((6, 128)) * 0.05).astype(np.float32),
            "wout": (rng.standard_normal(129) * 0.1).astype(np.float32)}


@pytest.mark.parametrize("W", [181, 336])
def test_filter_kernel_matches_torch(W):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(W)
    wts = _random_weights(rng)
    n = 7 * W + 55
    seq = "".join(rng.choice(list("ACGU"), n))
    dsq = cmfile.digitize(seq)
    d = torch.from_numpy(dsq).cuda()
    sc = L.Scanner(0)
    try:
        f = prefilter.Prefilter(sc, wts, W)
        logit, ms = f.logits(d.data_ptr(), 1, n)
        f.close()
    finally:
        sc.close()
    nwin = (n + W - 1) // W
    assert len(logit) == nwin and ms > 0
    wins = []
    for k in range(nwin):
        a = 1 + k * W
        body = dsq[a: min(a + 2 * W, n + 1)]
        w = np.full(2 * W + 2, 255, np.uint8)
        w[1: 1 + len(body)] = body
        w[1 + len(body):-1] = 4          # beyond the sequence: a non-ACGU code reads as zero input
        wins.append(w)
    ref = prefilter.reference_logits(wts, wins)
    assert np.all(np.abs(logit - ref) <= 0.05 + 0.02 * np.abs(ref)), (logit[:5], ref[:5])


def test_filter_heads_match_torch():
    """Three read-out heads on one trunk: every head's logits match the
    network in PyTorch, and head 0 equals the one-head filter bit for bit."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    W = 181
    wts = _random_weights(rng)
    heads = dict(wts)
    heads["wout"] = np.stack([wts["wout"]] + [(rng.standard_normal(129) * 0.1).astype(np.float32) for _ in range(2)])
    n = 5 * W + 17
    dsq = cmfile.digitize("".join(rng.choice(list("ACGU"), n)))
    d = torch.from_numpy(dsq).cuda()
    sc = L.Scanner(0)
    try:
        f1 = prefilter.Prefilter(sc, wts, W)
        one, _ = f1.logits(d.data_ptr(), 1, n)
        f1.close()
        f3 = prefilter.Prefilter(sc, heads, W)
        three, _ = f3.logits(d.data_ptr(), 1, n)
        f3.close()
    finally:
        sc.close()
    nwin = (n + W - 1) // W
    assert three.shape == (nwin, 3)
    assert np.array_equal(three[:, 0].view(np.uint32), one.view(np.uint32))
    wins = []
    for k in range(nwin):
        a = 1 + k * W
        body = dsq[a: min(a + 2 * W, n + 1)]
        w = np.full(2 * W + 2, 255, np.uint8)
        w[1: 1 + len(body)] = body
        w[1 + len(body):-1] = 4
        wins.append(w)
    ref = prefilter.reference_logits(heads, wins)
    assert ref.shape == (nwin, 3)
    assert np.all(np.abs(three - ref) <= 0.05 + 0.02 * np.abs(ref))


def test_dinuc_shuffle_preserves_doublets():
    rng = np.random.default_rng(1)
    s = "".join(rng.choice(list("ACGU"), 500))
    t = prefilter.dinuc_shuffle(s, rng)
    cnt = lambda x: sorted(a + b for a, b in zip(x[:-1], x[1:]))
    assert len(t) == len(s) and t[0] == s[0] and t[-1] == s[-1] and cnt(t) == cnt(s) and t != s
