"""Hand-written training of the pre-filter network (cmgb_filter_trainer_*).

1. One step's gradients against PyTorch autograd on the same weights and
   windows (FP32 on the CPU, with the kernels' BF16 rounding points in the
   forward pass: the dilated layers' weights and every layer's output).  The
   device backward also rounds each layer's input gradient to BF16 (the
   tensor-core operand type), so the comparison is a relative norm error per
   gradient tensor, bounded in the test.
2. A short training run on a motif task converges, and the trained weights
   load into the inference kernels (Prefilter) and classify held-out windows.
"""
import numpy as np
import pytest

from infernal_gb300 import cmfile, lib as L, prefilter

pytestmark = pytest.mark.gpu
DIL = (1, 2, 4, 8, 16, 32)


def _torch_grads(ws, wins, y, posw):
    import torch
    import torch.nn.functional as F
    bf = lambda t: t.to(torch.bfloat16).to(torch.float32)
    w0, w, bias, wout = [torch.tensor(a, dtype=torch.float32, requires_grad=True) for a in ws]
    B, n = wins.shape
    x = torch.zeros(B, 4, n)
    x[np.repeat(np.arange(B), n), wins.ravel().astype(np.int64), np.tile(np.arange(n), B)] = 1.0   # one-hot [B, 4, 2W]
    a = bf(F.relu(F.conv1d(x, w0.permute(2, 1, 0), bias[0], padding=4)))
    for l in range(1, 6):
        d = DIL[l]
        a = bf(F.relu(F.conv1d(a, bf(w[l - 1]).permute(1, 2, 0), bias[l], padding=4 * d, dilation=d)))
    pooled = a.max(dim=2).values
    if wout.dim() == 1:                    # one head: labels [B]
        z = pooled @ wout[:128] + wout[128]
        loss = F.binary_cross_entropy_with_logits(z, torch.tensor(y), pos_weight=torch.tensor(posw))
    else:                                  # [H][129]: labels [B][H], a pos weight per head, the heads' losses summed
        z = pooled @ wout[:, :128].T + wout[:, 128]
        loss = sum(F.binary_cross_entropy_with_logits(z[:, h], torch.tensor(y[:, h]), pos_weight=torch.tensor(posw[h]))
                   for h in range(wout.shape[0]))
    loss.backward()
    return float(loss), [t.grad.numpy() for t in (w0, w, bias, wout)]


@pytest.fixture(scope="module")
def gpu():
    s = L.Scanner(0)
    yield s
    s.close()


def test_gradients_match_autograd(gpu):
    W, B = 336, 8
    rng = np.random.default_rng(5)
    tr = prefilter.NativeTrainer(gpu, W, B, seed=3)
    try:
        wins = rng.integers(0, 4, (B, 2 * W)).astype(np.uint8)
        y = np.array([1, 0] * (B // 2), np.float32)
        ws = tr.get()
        loss, _ = tr.step(wins, y, 3.0, 0.0)
        _, gs = tr.get(grads=True)
    finally:
        tr.close()
    ref_loss, ref = _torch_grads(ws, wins, y, 3.0)
    assert abs(loss - ref_loss) < 1e-3 * max(1.0, abs(ref_loss))
    names = ("w0", "w", "bias", "wout")
    for name, g, r in zip(names, gs, ref):
        rel = np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-12)
        print(f"{name}: |g| {np.linalg.norm(r):.4g}, relative error {rel:.4f}")
        assert rel < (0.01 if name == "wout" else 0.05), name
    for l in range(5):                     # per dilated layer too
        rel = np.linalg.norm(gs[1][l] - ref[1][l]) / max(np.linalg.norm(ref[1][l]), 1e-12)
        assert rel < 0.05, l


def test_gradients_match_autograd_heads(gpu):
    """Three read-out heads on the one-head test's trunk and windows (same
    trainer seed, so the same arg-max cells), labels and positive weights per
    head: loss and gradients against PyTorch autograd with the one-head
    test's tolerances."""
    W, B, H = 336, 8, 3
    rng = np.random.default_rng(5)
    tr = prefilter.NativeTrainer(gpu, W, B, seed=3, heads=H)
    try:
        wins = rng.integers(0, 4, (B, 2 * W)).astype(np.uint8)
        y = np.stack([np.array([1, 0] * (B // 2), np.float32), (rng.random(B) < 0.5).astype(np.float32),
                      (rng.random(B) < 0.5).astype(np.float32)], axis=1)
        posw = np.array([3.0, 2.0, 0.5], np.float32)
        ws = tr.get()
        assert ws[3].shape == (H, 129)
        loss, _ = tr.step(wins, y, posw, 0.0)
        _, gs = tr.get(grads=True)
    finally:
        tr.close()
    ref_loss, ref = _torch_grads(ws, wins, y, posw)
    assert abs(loss - ref_loss) < 1e-3 * max(1.0, abs(ref_loss))
    for name, g, r in zip(("w0", "w", "bias", "wout"), gs, ref):
        rel = np.linalg.norm(g - r) / max(np.linalg.norm(r), 1e-12)
        print(f"{name}: relative error {rel:.4f}")
        assert rel < (0.01 if name == "wout" else 0.05), name


def test_identical_heads_repeat_the_one_head_network(gpu):
    """Three identical heads with identical labels and weights: every head's
    read-out gradient equals the one-head trainer's bit for bit (same
    forward, same per-window loss gradient), the loss is three times the
    one-head loss, and the trunk gradients are three times the one-head ones
    up to the BF16 rounding of the input gradients."""
    W, B = 128, 8
    rng = np.random.default_rng(8)
    wins = rng.integers(0, 4, (B, 2 * W)).astype(np.uint8)
    y = (rng.random(B) < 0.5).astype(np.float32)
    t1 = prefilter.NativeTrainer(gpu, W, B, seed=9)
    t3 = prefilter.NativeTrainer(gpu, W, B, seed=9, heads=3)
    try:
        w1 = t1.get()
        t3.set(w1[0], w1[1], w1[2], np.stack([w1[3]] * 3))
        l1, _ = t1.step(wins, y, 1.5, 0.0)
        l3, _ = t3.step(wins, np.repeat(y[:, None], 3, axis=1), 1.5, 0.0)
        _, g1 = t1.get(grads=True)
        _, g3 = t3.get(grads=True)
    finally:
        t1.close(); t3.close()
    assert abs(l3 - 3 * l1) <= 1e-5 * abs(3 * l1)
    for h in range(3):
        assert np.array_equal(g3[3][h].view(np.uint32), g1[3].view(np.uint32))
    for a, b in zip(g3[:3], g1[:3]):
        assert np.linalg.norm(a - 3 * b) <= 0.01 * np.linalg.norm(3 * b)


def _motif_batch(rng, B, W, motif):
    wins = rng.integers(0, 4, (B, 2 * W)).astype(np.uint8)
    y = (rng.random(B) < 0.5).astype(np.float32)
    for b in np.nonzero(y)[0]:
        p = int(rng.integers(0, 2 * W - len(motif)))
        wins[b, p:p + len(motif)] = motif
    return wins, y


def _motif_training(gpu, W, B, motif, steps=300):
    """The motif task from a fixed seed: (loss per step, fp32 weights, exported weights)."""
    rng = np.random.default_rng(11)
    tr = prefilter.NativeTrainer(gpu, W, B, seed=1)
    try:
        losses = []
        for it in range(steps):
            x, y = _motif_batch(rng, B, W, motif)
            loss, ms = tr.step(x, y, 1.0, 2e-3)
            losses.append(loss)
        return np.array(losses, np.float32), tr.get(), tr.weights(), ms
    finally:
        tr.close()


def test_training_converges_and_loads_into_inference(gpu):
    import torch
    W, B = 64, 64
    motif = np.array([2, 2, 2, 0, 1, 1, 1, 3, 0, 2], np.uint8)     # GGGACCCUAG
    losses, w32, wts, ms = _motif_training(gpu, W, B, motif)
    print(f"loss {losses[0]:.3f} -> {losses[-1]:.3f}; last step {ms:.2f} ms")
    # the trainer's reductions have a fixed order: a second run from the same
    # seed on the same batches repeats every loss and weight bit for bit
    losses2, w32b, _, _ = _motif_training(gpu, W, B, motif)
    print(f"second run: loss {losses2[0]:.3f} -> {losses2[-1]:.3f}")
    assert np.array_equal(losses.view(np.uint32), losses2.view(np.uint32))
    for a, b in zip(w32, w32b):
        assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert losses[-1] < 0.5 * losses[0]
    rng = np.random.default_rng(12)
    # held-out windows through the inference kernels: window k of a scan starts at 1 + kW
    x, y = _motif_batch(rng, 200, W, motif)
    seq = np.concatenate([[cmfile.DSQ_SENTINEL], x.ravel(), [cmfile.DSQ_SENTINEL]]).astype(np.uint8)
    f = prefilter.Prefilter(gpu, wts, W)
    try:
        d = torch.from_numpy(seq).cuda()
        logit, _ = f.logits(d.data_ptr(), 1, len(seq) - 2)
    finally:
        f.close()
    acc = float(((logit[0::2][:200] > 0) == (y > 0.5)).mean())
    print(f"held-out accuracy {acc:.3f}")
    assert acc > 0.9
