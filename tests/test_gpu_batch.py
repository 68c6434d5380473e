"""GPU batched scans (cmgb_ScanBatch): every sequence of a batch gets exactly
the result of the single-sequence scanner on that sequence -- hits (local
coordinates, modes), envelope, best score and best mode -- for all five
algorithms; a few sequences are also checked against the oracle."""
import zlib

import numpy as np
import pytest

import oracle
from infernal_gb300 import cmfile, emit, lib as L

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    s = L.Scanner(0)
    yield s
    s.close()


def _batch(m, rng, n, lo, hi, frac_hit=0.3):
    out = []
    for k in range(n):
        L_ = int(np.exp(rng.uniform(np.log(lo), np.log(hi))))
        bg = "".join(rng.choice(list("ACGU"), L_))
        if rng.random() < frac_hit:
            s = emit.sample(m, rng)
            a, b = sorted(int(x) for x in rng.integers(0, len(s) + 1, 2))
            frag = s[a:b] if b - a > 20 else s
            pos = int(rng.integers(0, max(1, L_ - len(frag))))
            bg = (bg[:pos] + frag + bg[pos + len(frag):])[:max(L_, len(frag))]
        out.append(cmfile.digitize(bg))
    return out


@pytest.mark.parametrize("name,algo,qdb,n,lo,hi", [
    ("Vault", "cyk", 1, 300, 100, 3000), ("Vault", "inside", 2, 120, 100, 2000), ("tRNA", "finside", 2, 100, 60, 1500),
    ("Plant_SRP", "cyk", 1, 80, 100, 2500), ("Plant_SRP", "trcyk", 1, 60, 100, 400), ("Vault", "trinside", 2, 60, 100, 400)])
def test_batch_equals_single_scans(gpu, models, name, algo, qdb, n, lo, hi):
    m = models[name]
    rng = np.random.default_rng(zlib.crc32(f"{name}{algo}batch".encode()))
    seqs = _batch(m, rng, n, lo, hi)
    gpu.set_shape(0, 0, 0)
    tr = algo.startswith("tr")
    passes = (2, 3, 4)
    for p in (passes if tr else (0,)):
        rs = gpu.scan_batch(m, seqs, algo=algo, qdbidx=qdb, pass_idx=p, cutoff=0.0, env_cutoff=2.0)
        assert len(rs) == n
        for q, d in enumerate(seqs):
            L_ = len(d) - 2
            if tr:
                s = gpu.tr_scan(m, d, 1, L_, algo=algo, qdbidx=qdb, pass_idx=p, cutoff=0.0, env_cutoff=2.0)
            else:
                s = gpu.scan(m, d, 1, L_, algo=algo, qdbidx=qdb, cutoff=0.0, env_cutoff=2.0)
            assert rs[q].hits == s.hits
            assert (rs[q].envi, rs[q].envj) == (s.envi, s.envj)
            assert np.float32(rs[q].sc) == np.float32(s.sc)
            if tr:
                assert rs[q].mode == s.mode
    assert gpu.last_launches() >= 1


def test_batch_vs_oracle(gpu, models):
    m = models["tRNA"]
    rng = np.random.default_rng(77)
    seqs = _batch(m, rng, 8, 50, 400, frac_hit=0.6)
    for algo, qdb in (("cyk", 1), ("trinside", 2)):
        rs = gpu.scan_batch(m, seqs, algo=algo, qdbidx=qdb, pass_idx=4, cutoff=0.0, env_cutoff=1.0, notgreedy=True)
        for q, d in enumerate(seqs):
            if algo == "cyk":
                o = oracle.scan(m, d, 1, len(d) - 2, algo=algo, qdbidx=qdb, cutoff=0.0, env_cutoff=1.0, notgreedy=True)
            else:
                o = oracle.tr_scan(m, d, 1, len(d) - 2, algo=algo, qdbidx=qdb, pass_idx=4, cutoff=0.0, env_cutoff=1.0,
                                   notgreedy=True)
                assert rs[q].mode == o[5]
            assert rs[q].hits == o[0] and (rs[q].envi, rs[q].envj) == (o[1], o[2])
            assert np.float32(rs[q].sc) == np.float32(o[3])


def test_batch_contract_errors(gpu, models):
    m = models["tRNA"]
    d = cmfile.digitize("ACGU" * 20)
    with pytest.raises(L.ScanError) as e:
        gpu.scan_batch(m, [d], algo="trcyk", pass_idx=1)
    assert e.value.status == 11
    lib = gpu.lib
    import ctypes
    err = ctypes.create_string_buffer(256)
    offs = np.array([0], np.int64)
    lens = np.array([500], np.int64)            # runs past the end of the buffer
    st = lib.cmgb_ScanBatch(gpu._ctx, gpu.model(m), err, 0, 1, 0, d.ctypes.data, len(d), offs.ctypes.data,
                            lens.ctypes.data, 1, 0.0, None, 0, 0.0, None, None, None, None, None)
    assert st == 10 and b"outside the buffer" in err.value


def test_explicit_ctas_per_sm_with_large_shared_memory(models):
    """A launch shape with an explicit CTA count still sets each kernel's
    dynamic shared-memory limit: a truncated batch whose 32-row plan needs
    about 90 KB of shared memory, at one CTA per SM, equals the default
    launch."""
    m = models["Plant_SRP"]
    rng = np.random.default_rng(zlib.crc32(b"explicit-cps"))
    reads = [cmfile.digitize("".join(rng.choice(list("ACGU"), int(rng.integers(150, 301))))) for _ in range(24)]
    reads[3] = cmfile.digitize(emit.sample(m, rng)[40:])
    s = L.Scanner(0)
    try:
        out = []
        for cps in (0, 1):
            s.set_shape(32, 0, cps, 0, 2)
            rs = s.scan_batch(m, reads, algo="trcyk", qdbidx=1, pass_idx=4, cutoff=5.0, env_cutoff=5.0)
            out.append([(r.hits, r.envi, r.envj, np.float32(r.sc).view(np.uint32)) for r in rs])
        assert out[0] == out[1]
        assert any(h for h, _, _, _ in out[0])
    finally:
        s.close()
