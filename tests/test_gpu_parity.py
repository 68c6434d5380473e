"""GPU parity: the sm_103a scanners against the reference's golden vectors and
the CPU oracle, through the C ABI.  CYK, integer Inside, hit lists (greedy and
optimal resolution, NULL3), envelopes, best scores and per-state best scores
must all be bit-identical."""
import zlib

import numpy as np
import pytest

import oracle
from conftest import hits_from_golden
from infernal_gb300 import cmfile, lib as L

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gpu():
    s = L.Scanner(0)
    yield s
    s.close()


def _check(r, hits, ei, ej, sc, vsc):
    assert r.hits == hits
    assert (r.envi, r.envj) == (ei, ej)
    assert np.float32(r.sc) == np.float32(sc)
    if vsc is not None:
        assert np.array_equal(r.vsc.view(np.int32), np.asarray(vsc, np.float32).view(np.int32))


@pytest.mark.parametrize("T,arena", [(16, 1), (5, 1), (48, 2), (128, 2)])
def test_golden_on_gpu(gpu, golden, models, T, arena):
    """Shared-memory tiles (arena 1) and the global-memory tile arena (arena 2)."""
    meta, arrays = golden
    gpu.set_shape(T, 0, 0, 0, arena)
    n = 0
    for c in meta:
        if c["algo"] not in ("cyk", "refcyk", "inside", "finside"):
            continue
        algo = "cyk" if c["algo"] == "refcyk" else c["algo"]
        r = gpu.scan(models[c["model"]], arrays["dsq." + c["seq"]], c["i0"], c["j0"], algo=algo, qdbidx=c["qdbidx"],
                     cutoff=c["cutoff"], do_null3=bool(c["null3"]), env_cutoff=c["env_cutoff"],
                     notgreedy=bool(c["notgreedy"]), want_vsc=True)
        _check(r, hits_from_golden(c), c["envi"], c["envj"], float.fromhex(c["sc"]), arrays[f"vsc.{c['id']}"])
        n += 1
    assert n >= 40
    assert gpu.last_launches() >= 1


@pytest.mark.parametrize("name,algo,qdb", [("tRNA", "cyk", 1), ("Vault", "cyk", 1), ("Plant_SRP", "cyk", 1),
                                           ("tRNA", "inside", 2), ("Vault", "inside", 2), ("Plant_SRP", "inside", 2),
                                           ("Vault", "finside", 2)])
def test_random_targets_vs_oracle(gpu, models, name, algo, qdb):
    m = models[name]
    rng = np.random.default_rng(zlib.crc32(f"{name}{algo}".encode()))
    n = 20000 if algo == "cyk" else 8000
    if name == "Plant_SRP":
        n //= 2
    dsq = cmfile.digitize("".join(rng.choice(list("ACGU"), n, p=[0.3, 0.2, 0.2, 0.3])))
    gpu.set_shape(0, 0, 0)
    for i0, j0 in ((1, n), (999, n - 77)):
        r = gpu.scan(m, dsq, i0, j0, algo=algo, qdbidx=qdb, cutoff=0.0, env_cutoff=3.0, want_vsc=True)
        o = oracle.scan(m, dsq, i0, j0, algo=algo, qdbidx=qdb, cutoff=0.0, env_cutoff=3.0)
        _check(r, *o)


def test_window_and_tile_invariance(gpu, models):
    """Window length, tile rows and CTA count change only the schedule."""
    m = models["Vault"]
    rng = np.random.default_rng(5)
    n = 60000
    dsq = cmfile.digitize("".join(rng.choice(list("ACGU"), n)))
    ref = None
    for T, win, cps, nt, ar in ((16, 0, 0, 0, 1), (8, 1500, 1, 256, 1), (3, 4000, 2, 0, 1), (16, 777, 1, 0, 2),
                                (64, 2500, 0, 0, 2), (33, 0, 0, 128, 2), (96, 3000, 0, 0, 2), (128, 0, 0, 0, 2)):
        gpu.set_shape(T, win, cps, nt, ar)
        r = gpu.scan(m, dsq, 1, n, algo="cyk", qdbidx=1, cutoff=-1.0, env_cutoff=3.0, want_vsc=True)
        key = (r.hits, r.envi, r.envj, r.sc, r.vsc.tobytes())
        assert ref is None or key == ref
        ref = key
    gpu.set_shape(0, 0, 0)


def test_device_resident_entry_point(gpu, models):
    torch = pytest.importorskip("torch")
    m = models["tRNA"]
    rng = np.random.default_rng(9)
    n = 5000
    dsq = cmfile.digitize("".join(rng.choice(list("ACGU"), n)))
    d = torch.from_numpy(dsq).cuda()
    torch.cuda.synchronize()
    for algo, q in (("cyk", 1), ("inside", 2)):
        a = gpu.scan(m, dsq, 1, n, algo=algo, qdbidx=q, env_cutoff=2.0)
        b = gpu.scan(m, None, 1, n, algo=algo, qdbidx=q, env_cutoff=2.0, device_ptr=d.data_ptr())
        assert (a.hits, a.envi, a.envj, a.sc) == (b.hits, b.envi, b.envj, b.sc)


def test_contract_errors_on_gpu(gpu, models):
    m = models["tRNA"]
    dsq = cmfile.digitize("ACGU" * 40)
    with pytest.raises(L.ScanError) as e:
        gpu.scan(m, dsq, 100, 10)
    assert e.value.status == 10


def test_autotune_keeps_results(gpu, models):
    """The autotuner only changes the schedule: results before and after tuning agree."""
    m = models["Vault"]
    rng = np.random.default_rng(21)
    n = 30000
    dsq = cmfile.digitize("".join(rng.choice(list("ACGU"), n)))
    gpu.set_shape(0, 0, 0)
    a = gpu.scan(m, dsq, 1, n, algo="inside", qdbidx=2, cutoff=0.0, env_cutoff=2.0, want_vsc=True)
    T, arena = gpu.autotune(m, 2, "inside", 20000)
    assert T in (16, 32, 48, 64, 96, 128) and arena in (1, 2)
    b = gpu.scan(m, dsq, 1, n, algo="inside", qdbidx=2, cutoff=0.0, env_cutoff=2.0, want_vsc=True)
    assert (a.hits, a.envi, a.envj, a.sc, a.vsc.tobytes()) == (b.hits, b.envi, b.envj, b.sc, b.vsc.tobytes())
