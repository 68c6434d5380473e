"""GPU parity of the truncated scanners (cmgb_RefTrCYKScan /
cmgb_RefITrInsideScan) against the reference's golden vectors and the CPU
oracle, through the C ABI: hits (with their modes), envelope, best score, the
best parse's mode and per-state best scores must be bit-identical."""
import zlib

import numpy as np
import pytest

import oracle
from conftest import hits_from_golden
from infernal_gb300 import cmfile, emit, lib as L

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    s = L.Scanner(0)
    yield s
    s.close()


def _check(r, o):
    hits, ei, ej, sc, vsc, mode = o
    assert r.hits == hits
    assert (r.envi, r.envj) == (ei, ej)
    assert np.float32(r.sc) == np.float32(sc)
    assert r.mode == mode
    if r.vsc is not None:
        assert np.array_equal(r.vsc.view(np.int32), np.asarray(vsc, np.float32).view(np.int32))


@pytest.mark.parametrize("T,win,arena", [(16, 0, 1), (7, 0, 1), (32, 0, 2), (8, 64, 1)])
def test_tr_golden_on_gpu(gpu, golden, models, T, win, arena):
    """Every truncated golden case; win=64 splits the targets into many windows,
    which exercises the host's cross-window root test."""
    meta, arrays = golden
    gpu.set_shape(T, win, 0, 0, arena)
    n = 0
    for c in meta:
        if c["algo"] not in ("trcyk", "trinside"):
            continue
        r = gpu.tr_scan(models[c["model"]], arrays["dsq." + c["seq"]], c["i0"], c["j0"], algo=c["algo"],
                        qdbidx=c["qdbidx"], pass_idx=c["pass_idx"], cutoff=c["cutoff"], do_null3=bool(c["null3"]),
                        env_cutoff=c["env_cutoff"], notgreedy=bool(c["notgreedy"]), want_vsc=True)
        _check(r, (hits_from_golden(c), c["envi"], c["envj"], float.fromhex(c["sc"]), arrays[f"vsc.{c['id']}"], c["mode"]))
        n += 1
    assert n >= 60
    gpu.set_shape(0, 0, 0)


def _reads(m, rng, nreads, L=(100, 400)):
    """Reads as the truncated passes see them: emitted sequences cut at random
    5'/3' points, padded with background, plus pure background reads."""
    out = []
    for k in range(nreads):
        n = int(rng.integers(*L))
        bg = "".join(rng.choice(list("ACGU"), n))
        if k % 3 == 2:
            out.append(bg)
            continue
        s = emit.sample(m, rng)
        a, b = sorted(int(x) for x in rng.integers(0, len(s) + 1, 2))
        frag = s[a:b] if b - a > 10 else s
        out.append((frag + bg)[:n] if k % 3 == 0 else (bg + frag)[-n:])
    return out


@pytest.mark.parametrize("name,algo,qdb", [("tRNA", "trcyk", 1), ("Vault", "trcyk", 1), ("Plant_SRP", "trcyk", 1),
                                           ("tRNA", "trinside", 2), ("Vault", "trinside", 2), ("Plant_SRP", "trinside", 2)])
def test_reads_vs_oracle(gpu, models, name, algo, qdb):
    m = models[name]
    rng = np.random.default_rng(zlib.crc32(f"{name}{algo}tr".encode()))
    gpu.set_shape(0, 0, 0)
    for k, seq in enumerate(_reads(m, rng, 6)):
        dsq = cmfile.digitize(seq)
        p = (2, 3, 4)[k % 3]
        r = gpu.tr_scan(m, dsq, 1, len(seq), algo=algo, qdbidx=qdb, pass_idx=p, cutoff=0.0, env_cutoff=2.0, want_vsc=True)
        o = oracle.tr_scan(m, dsq, 1, len(seq), algo=algo, qdbidx=qdb, pass_idx=p, cutoff=0.0, env_cutoff=2.0)
        _check(r, o)


@pytest.mark.parametrize("algo", ["trcyk", "trinside"])
def test_long_target_many_windows(gpu, models, algo):
    """A target many windows long: the running-maximum root test crosses windows."""
    m = models["Vault"]
    rng = np.random.default_rng(33)
    n = 6000 if algo == "trcyk" else 3000
    seq = "".join(rng.choice(list("ACGU"), n))
    ins = emit.sample(m, rng)
    seq = seq[:2000] + ins + seq[2000 + len(ins):]
    dsq = cmfile.digitize(seq)
    o = oracle.tr_scan(m, dsq, 1, n, algo=algo, qdbidx=1, pass_idx=4, cutoff=0.0, env_cutoff=2.0)
    for T, win, ar in ((16, 0, 1), (8, 200, 1), (16, 512, 2)):
        gpu.set_shape(T, win, 0, 0, ar)
        r = gpu.tr_scan(m, dsq, 1, n, algo=algo, qdbidx=1, pass_idx=4, cutoff=0.0, env_cutoff=2.0, want_vsc=True)
        _check(r, o)
    gpu.set_shape(0, 0, 0)


def test_tr_device_resident_entry_point(gpu, models):
    torch = pytest.importorskip("torch")
    m = models["tRNA"]
    rng = np.random.default_rng(19)
    seq = _reads(m, rng, 1)[0]
    dsq = cmfile.digitize(seq)
    d = torch.from_numpy(dsq).cuda()
    torch.cuda.synchronize()
    for algo in ("trcyk", "trinside"):
        a = gpu.tr_scan(m, dsq, 1, len(seq), algo=algo, pass_idx=4, env_cutoff=2.0)
        b = gpu.tr_scan(m, None, 1, len(seq), algo=algo, pass_idx=4, env_cutoff=2.0, device_ptr=d.data_ptr())
        assert (a.hits, a.envi, a.envj, a.sc, a.mode) == (b.hits, b.envi, b.envj, b.sc, b.mode)


def test_tr_contract_errors_on_gpu(gpu, models):
    m = models["tRNA"]
    dsq = cmfile.digitize("ACGU" * 40)
    for bad in (0, 1, 6):   # cm_TrFillFromPassIdx rejects these passes with eslEINVAL
        with pytest.raises(L.ScanError) as e:
            gpu.tr_scan(m, dsq, 1, 100, pass_idx=bad)
        assert e.value.status == 11
    with pytest.raises(L.ScanError) as e:
        gpu.tr_scan(m, dsq, 100, 10, pass_idx=4)
    assert e.value.status == 10
    with pytest.raises(L.ScanError) as e:
        gpu.tr_scan(m, dsq, 1, 100, qdbidx=3, pass_idx=4)
    assert e.value.status == 10
