"""Multi-model batched scans (cmgb_ScanMulti): every (model, sequence) job of
one launch gets exactly the result cmgb_ScanBatch gives for that model over
that sequence -- hits (local coordinates), envelope and best score.  The CPU
tests run the kernel source in the host emulation on small cases; the GPU
tests mix three models (shared-memory and global-memory plans) over sequences
of uneven length."""
import zlib

import numpy as np
import pytest

from infernal_gb300 import cmfile, emit, lib as L


def _seqs(models, rng, n, lo, hi, frac_hit=0.4):
    out = []
    for k in range(n):
        L_ = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        bg = "".join(rng.choice(list("ACGU"), L_))
        if rng.random() < frac_hit:
            s = emit.sample(models[int(rng.integers(len(models)))], rng)
            pos = int(rng.integers(0, max(1, L_ - len(s))))
            bg = (bg[:pos] + s + bg[pos + len(s):])[:max(L_, len(s))]
        out.append(cmfile.digitize(bg))
    return out


def _check(sc, ms, seqs, jobs, algo, qdb, cutoffs):
    rs = sc.scan_multi(ms, seqs, jobs=jobs, algo=algo, qdbidx=qdb, cutoffs=cutoffs, env_cutoff=2.0)
    assert len(rs) == len(jobs)
    want = {}
    for mi, m in enumerate(ms):
        qs = sorted({q for a, q in jobs if a == mi})
        if not qs:
            continue
        bs = sc.scan_batch(m, [seqs[q] for q in qs], algo=algo, qdbidx=qdb, cutoff=cutoffs[mi], env_cutoff=2.0)
        for q, b in zip(qs, bs):
            want[(mi, q)] = b
    nh = 0
    for r, job in zip(rs, jobs):
        b = want[job]
        assert r.hits == b.hits, job
        assert (r.envi, r.envj) == (b.envi, b.envj), job
        assert np.float32(r.sc) == np.float32(b.sc), job
        nh += len(r.hits)
    return nh


def test_multi_equals_batch_emulated(emu, models):
    ms = [models["tRNA"], models["Vault"]]
    rng = np.random.default_rng(31)
    seqs = _seqs(ms, rng, 2, 40, 80)
    jobs = [(0, 0), (1, 1), (1, 0)]
    _check(emu, ms, seqs, jobs, "cyk", 1, [0.0, 2.0])


def test_multi_sparse_jobs_inside_emulated(emu, models):
    ms = [models["tRNA"], models["Vault"]]
    rng = np.random.default_rng(32)
    seqs = _seqs(ms, rng, 3, 40, 80)
    _check(emu, ms, seqs, [(1, 2), (0, 0)], "inside", 2, [0.0, 0.0])


def test_multi_rejects_repeated_pairs(emu, models):
    ms = [models["tRNA"]]
    seqs = [cmfile.digitize("ACGU" * 30)]
    with pytest.raises(L.ScanError):
        emu.scan_multi(ms, seqs, jobs=[(0, 0), (0, 0)], algo="cyk", qdbidx=1)
    with pytest.raises(ValueError):
        emu.scan_multi(ms, seqs, algo="trcyk")


@pytest.fixture(scope="module")
def gpu():
    s = L.Scanner(0)
    yield s
    s.close()


@pytest.mark.gpu
@pytest.mark.parametrize("algo,qdb", [("cyk", 1), ("inside", 2), ("finside", 2)])
def test_multi_equals_batch_gpu(gpu, models, algo, qdb):
    ms = [models["tRNA"], models["Vault"], models["Plant_SRP"]]
    rng = np.random.default_rng(zlib.crc32(f"multi{algo}".encode()))
    seqs = _seqs(ms, rng, 40, 100, 5000)
    gpu.set_shape(0, 0, 0)
    jobs = [(a, q) for a in range(3) for q in range(40)]
    nh = _check(gpu, ms, seqs, jobs, algo, qdb, [0.0, 0.0, 0.0])
    assert nh > 0
    assert gpu.last_launches() >= 1
    # a job subset in shuffled order
    sub = [jobs[k] for k in rng.permutation(len(jobs))[:50]]
    _check(gpu, ms, seqs, sub, algo, qdb, [3.0, 0.0, 5.0])


def _overlapping_regions_case(models, rng, n=6000):
    """One residue buffer of n residues and, per model, its own
    non-overlapping regions; regions of different models overlap."""
    body = "".join(rng.choice(list("ACGU"), n))
    for k, m in enumerate(models):
        e = emit.sample(m, rng)
        pos = n // 12 + (3 * n // 10) * k
        body = body[:pos] + e + body[pos + len(e):]
    buf = cmfile.digitize(body[:n])
    spans = []                                  # (model, offset, length)
    for k in range(len(models)):
        spans += [(k, 0, 5 * n // 12), (k, 13 * n // 30 + (n // 60) * k, n // 2 - (n // 60) * k)]
    spans += [(0, n - n // 20, n // 24)]
    return buf, spans


def test_multi_overlapping_regions_emulated(emu, models):
    """Per-model regions that overlap across models: each candidate goes to
    the job of its own model; every job equals the model's batch scan of the
    same region."""
    ms = [models["tRNA"], models["Vault"]]
    buf, spans = _overlapping_regions_case(ms, np.random.default_rng(31), n=1200)
    offs = np.array([o for _, o, _ in spans], np.int64)
    lens = np.array([n for _, _, n in spans], np.int64)
    jobs = [(k, q) for q, (k, _, _) in enumerate(spans)]
    rs = emu.scan_multi(ms, None, jobs=jobs, algo="cyk", qdbidx=1, cutoffs=[0.0, 0.0], env_cutoff=2.0, ranges=(buf, offs, lens))
    for (k, q), r in zip(jobs, rs):
        b = emu.scan_batch(ms[k], None, algo="cyk", qdbidx=1, cutoff=0.0, env_cutoff=2.0, ranges=(buf, offs[q:q + 1], lens[q:q + 1]))
        assert r.hits == b[0].hits and (r.envi, r.envj, r.sc) == (b[0].envi, b[0].envj, b[0].sc)
    assert sum(len(r.hits) for r in rs) > 0


@pytest.mark.gpu
def test_multi_device_buffer_equals_host_buffer_gpu(gpu, models):
    """cmgb_ScanMulti_dev (residues already in device memory, NULL3 on) equals
    cmgb_ScanMulti on the same overlapping per-model regions."""
    torch = pytest.importorskip("torch")
    ms = [models["tRNA"], models["Vault"], models["Plant_SRP"]]
    buf, spans = _overlapping_regions_case(ms, np.random.default_rng(32))
    offs = np.array([o for _, o, _ in spans], np.int64)
    lens = np.array([n for _, _, n in spans], np.int64)
    jobs = [(k, q) for q, (k, _, _) in enumerate(spans)]
    d = torch.from_numpy(buf).cuda()
    torch.cuda.synchronize()
    host = gpu.scan_multi(ms, None, jobs=jobs, algo="cyk", qdbidx=1, cutoffs=[0.0] * 3, env_cutoff=2.0, ranges=(buf, offs, lens))
    dev = gpu.scan_multi(ms, None, jobs=jobs, algo="cyk", qdbidx=1, cutoffs=[0.0] * 3, env_cutoff=2.0,
                         ranges=(None, offs, lens), device_buf=(d.data_ptr(), len(buf)))
    assert [r.hits for r in host] == [r.hits for r in dev]
    assert [(r.envi, r.envj, r.sc) for r in host] == [(r.envi, r.envj, r.sc) for r in dev]
    assert sum(len(r.hits) for r in host) > 0


@pytest.mark.gpu
def test_multi_autotuned_shapes_gpu(gpu, models):
    """Models tuned to different tile shapes and placements share a launch."""
    ms = [models["tRNA"], models["Vault"], models["Plant_SRP"]]
    for m in ms:
        gpu.autotune(m, 1, "cyk", sample_len=60000)
    rng = np.random.default_rng(77)
    seqs = _seqs(ms, rng, 30, 200, 4000)
    jobs = [(a, q) for a in range(3) for q in range(30)]
    _check(gpu, ms, seqs, jobs, "cyk", 1, [0.0, 0.0, 0.0])


def test_multi_and_calibrate_argument_checks(emu, models):
    """Contract violations return an error status before any device work."""
    import ctypes
    m = models["tRNA"]
    seqs = [cmfile.digitize("ACGU" * 30)]
    with pytest.raises(L.ScanError):                       # model index out of range
        emu.scan_multi([m], seqs, jobs=[(1, 0)], algo="cyk", qdbidx=1)
    with pytest.raises(L.ScanError):                       # sequence index out of range
        emu.scan_multi([m], seqs, jobs=[(0, 3)], algo="cyk", qdbidx=1)
    with pytest.raises(L.ScanError):                       # band set out of range
        emu.scan_multi([m], seqs, algo="cyk", qdbidx=3)
    # a sequence that does not fit its buffer (sentinel, residues, sentinel)
    lib = emu.lib
    mh = emu.model(m)
    buf = np.ascontiguousarray(seqs[0])
    offs, lens = np.array([0], np.int64), np.array([len(buf)], np.int64)
    jm, js = np.zeros(1, np.int32), np.zeros(1, np.int32)
    cut = np.zeros(1, np.float32)
    harr = (ctypes.c_void_p * 1)(mh.value)
    err = ctypes.create_string_buffer(256)
    st = lib.cmgb_ScanMulti(emu._ctx, harr, 1, cut.ctypes.data, err, 0, 1, buf.ctypes.data, len(buf), offs.ctypes.data,
                            lens.ctypes.data, 1, jm.ctypes.data, js.ctypes.data, 1, None, 1, 0.0, None, None, None, None)
    assert st == 10 and b"outside the buffer" in err.value
    # calibration: sizes and algorithm (float Inside is not a calibrated mode)
    e2 = L.ExpInfo()
    for algo, total, seqlen, tail in ((0, 500, 100, 750), (0, 10_000, 50, 750), (2, 10_000, 1000, 750), (0, 10_000, 1000, 0)):
        st = lib.cmgb_Calibrate(emu._ctx, mh, err, algo, total, seqlen, 1, tail, ctypes.byref(e2), None)
        assert st == 11, (algo, total, seqlen, tail)


def test_trainer_fails_loudly_without_a_gpu(emu):
    """The emulation build has no tensor cores: the trainer refuses instead of
    falling back to anything."""
    import ctypes
    h = ctypes.c_void_p()
    err = ctypes.create_string_buffer(256)
    st = emu.lib.cmgb_filter_trainer_create(emu._ctx, 64, 8, 1, ctypes.byref(h), err)
    assert st == 30 and not h.value and b"not available" in err.value
