"""Glocal-mode scans (no local begins or ends; cmsearch -g) against the
golden vectors written by the reference's own scanners
(tests/golden/gen_glocal.py): the oracle and the emulated kernel on the CPU,
every case on the GPU, bit for bit (hits, envelope, best score, per-state
best scores)."""
import json
import os

import numpy as np
import pytest

import oracle
from conftest import hits_from_golden
from infernal_gb300 import cmfile, lib as L

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def glocal():
    with open(os.path.join(HERE, "golden_glocal.json")) as fh:
        meta = json.load(fh)
    arrays = dict(np.load(os.path.join(HERE, "golden_glocal.npz")))
    models = {n: cmfile.load_npz(os.path.join(HERE, f"{n}.glocal.model.npz")) for n in ("tRNA", "Vault", "Plant_SRP")}
    return meta, arrays, models


def _check(hits, ei, ej, sc, vsc, c, arrays):
    assert hits == hits_from_golden(c)
    assert (ei, ej) == (c["envi"], c["envj"])
    assert np.float32(sc) == np.float32(float.fromhex(c["sc"]))
    assert np.array_equal(np.asarray(vsc, np.float32).view(np.int32), arrays[f"vsc.{c['id']}"].view(np.int32))


def test_glocal_models_have_no_local_begins_or_ends(glocal):
    _, _, models = glocal
    for m in models.values():
        assert (m.flags & 3) == 0
        assert np.all(m.endsc[m.sttype != cmfile.E_st] <= cmfile.IMPOSSIBLE)


def test_oracle_matches_reference_glocal(glocal):
    meta, arrays, models = glocal
    assert len(meta) >= 18
    for c in meta:
        r = oracle.scan(models[c["model"]], arrays["dsq." + c["seq"]], c["i0"], c["j0"], algo=c["algo"],
                        qdbidx=c["qdbidx"], cutoff=c["cutoff"], do_null3=bool(c["null3"]), env_cutoff=c["env_cutoff"])
        _check(*r, c, arrays)


def test_emulated_kernel_matches_reference_glocal(emu, glocal):
    meta, arrays, models = glocal
    n = 0
    for c in meta:
        if not c["seq"].endswith(".short") or c["model"] == "Plant_SRP":   # Plant_SRP: oracle and GPU legs only
            continue
        r = emu.scan(models[c["model"]], arrays["dsq." + c["seq"]], c["i0"], c["j0"], algo=c["algo"], qdbidx=c["qdbidx"],
                     cutoff=c["cutoff"], do_null3=bool(c["null3"]), env_cutoff=c["env_cutoff"], want_vsc=True)
        _check(r.hits, r.envi, r.envj, r.sc, r.vsc, c, arrays)
        n += 1
    assert n >= 4


@pytest.mark.gpu
@pytest.mark.parametrize("T,arena", [(16, 1), (48, 2)])
def test_glocal_on_gpu(glocal, T, arena):
    meta, arrays, models = glocal
    s = L.Scanner(0)
    try:
        s.set_shape(T, 0, 0, 0, arena)
        for c in meta:
            r = s.scan(models[c["model"]], arrays["dsq." + c["seq"]], c["i0"], c["j0"], algo=c["algo"], qdbidx=c["qdbidx"],
                       cutoff=c["cutoff"], do_null3=bool(c["null3"]), env_cutoff=c["env_cutoff"], want_vsc=True)
            _check(r.hits, r.envi, r.envj, r.sc, r.vsc, c, arrays)
    finally:
        s.close()
