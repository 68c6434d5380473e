"""CPU tests of the truncated scanners' C ABI: the truncated kernel source,
compiled for the test-only host-thread emulation of a CTA, reproduces the
oracle bit for bit -- including a target split into many windows, where the
host's cross-window root test decides which cells are reported -- and keeps
the reference's error behaviour.  No GPU is used.  Sequences are short: the
emulation runs every CUDA thread as an OS thread."""
import copy

import numpy as np
import pytest

import oracle
from infernal_gb300 import cmfile, emit, lib as L


def _target(m, seed, bg=20):
    rng = np.random.default_rng(seed)
    s = emit.sample(m, rng)
    return s[len(s) // 2:] + "".join(rng.choice(list("ACGU"), bg))


@pytest.mark.parametrize("name,algo,pidx,qdb,T,win,arena,ng", [
    ("tRNA", "trcyk", 4, 1, 8, 0, 1, 0), ("tRNA", "trinside", 3, 2, 8, 16, 2, 0), ("tRNA", "trcyk", 2, 0, 16, 24, 2, 1),
    ("tRNA", "trcyk", 3, 1, 5, 0, 1, 0), ("Vault", "trcyk", 4, 2, 12, 30, 2, 0)])
def test_emulated_tr_kernel_matches_oracle(emu, models, name, algo, pidx, qdb, T, win, arena, ng):
    m = models[name]
    seq = _target(m, 7)
    dsq = cmfile.digitize(seq)
    n = len(seq)
    emu.set_shape(T, win, 1, 0, arena)
    r = emu.tr_scan(m, dsq, 1, n, algo=algo, qdbidx=qdb, pass_idx=pidx, cutoff=-2.0, env_cutoff=1.0,
                    want_vsc=True, notgreedy=bool(ng))
    o = oracle.tr_scan(m, dsq, 1, n, algo=algo, qdbidx=qdb, pass_idx=pidx, cutoff=-2.0, env_cutoff=1.0,
                       notgreedy=bool(ng))
    assert r.hits == o[0]
    assert (r.envi, r.envj) == (o[1], o[2])
    assert np.float32(r.sc) == np.float32(o[3]) and r.mode == o[5]
    assert np.array_equal(r.vsc.view(np.int32), o[4].view(np.int32))
    emu.set_shape(0, 0, 0)


def test_tr_contract_errors(emu, models):
    m = models["tRNA"]
    dsq = cmfile.digitize("ACGU" * 10)
    with pytest.raises(L.ScanError) as e:
        emu.tr_scan(m, dsq, 1, 40, pass_idx=1)
    assert e.value.status == 11 and "pass idx" in str(e.value)
    with pytest.raises(L.ScanError) as e:
        emu.tr_scan(m, dsq, 30, 10, pass_idx=4)
    assert e.value.status == 10
    bare = copy.copy(m)                      # a model without truncation tables
    bare.tr_g_pty = None
    with pytest.raises(L.ScanError) as e:
        emu.tr_scan(bare, dsq, 1, 40, pass_idx=4)
    assert e.value.status == 10 and "truncation" in str(e.value)
