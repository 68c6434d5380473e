"""The nine panel CMs (tests/golden/panel: 227-960 states, 0-7
bifurcations, W 89-408) against golden vectors written by the reference's
own FastCYKScan (QDB1) and FastIInsideScan (QDB2) on seeded 4.4 kb targets
with emitted sequences embedded (tests/golden/gen_panel_golden.py): the
oracle on the CPU, the kernel source in the host emulation, the GPU scanners
in both tile placements, bit for bit."""
import json
import os

import numpy as np
import pytest

import oracle
from conftest import hits_from_golden
from infernal_gb300 import cmfile, lib as L

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def panel():
    with open(os.path.join(HERE, "golden_panel.json")) as fh:
        meta = json.load(fh)
    arrays = dict(np.load(os.path.join(HERE, "golden_panel.npz")))
    models = {c["model"]: cmfile.load_npz(os.path.join(HERE, "panel", f"{c['model']}.model.npz")) for c in meta}
    return meta, arrays, models


def _check(hits, ei, ej, sc, vsc, c, arrays):
    assert hits == hits_from_golden(c), c["model"]
    assert (ei, ej) == (c["envi"], c["envj"])
    assert np.float32(sc) == np.float32(float.fromhex(c["sc"]))
    assert np.array_equal(np.asarray(vsc, np.float32).view(np.int32), arrays[f"vsc.{c['id']}"].view(np.int32))


@pytest.mark.parametrize("k", range(18))
def test_panel_oracle_matches_reference(panel, k):
    meta, arrays, models = panel
    c = meta[k]
    if c["algo"] == "inside" and c["model"] in ("srp-euk", "rnaseP-eubact", "Cobalamin"):
        pytest.skip("the largest models' Inside cases run on the GPU leg only (CPU time)")
    r = oracle.scan(models[c["model"]], arrays["dsq." + c["seq"]], c["i0"], c["j0"], algo=c["algo"], qdbidx=c["qdbidx"],
                    cutoff=c["cutoff"], do_null3=bool(c["null3"]), env_cutoff=c["env_cutoff"])
    _check(*r, c, arrays)


@pytest.mark.parametrize("T,arena", [(24, 2), (128, 2)])
def test_panel_emulated_kernel_matches_reference(panel, emu, T, arena):
    """The scan kernel's source, run by the host-thread emulation of a CTA,
    on every panel case: hits, envelope, best score and per-state scores bit
    for bit against the reference's own output."""
    meta, arrays, models = panel
    emu.set_shape(T, 0, 1, 0, arena)
    try:
        for c in meta:
            r = emu.scan(models[c["model"]], arrays["dsq." + c["seq"]], c["i0"], c["j0"], algo=c["algo"], qdbidx=c["qdbidx"],
                         cutoff=c["cutoff"], do_null3=bool(c["null3"]), env_cutoff=c["env_cutoff"], want_vsc=True)
            _check(r.hits, r.envi, r.envj, r.sc, r.vsc, c, arrays)
    finally:
        emu.set_shape(0, 0, 0)


@pytest.mark.gpu
@pytest.mark.parametrize("T,arena", [(16, 1), (48, 2), (128, 2)])
def test_panel_on_gpu(panel, T, arena):
    meta, arrays, models = panel
    s = L.Scanner(0)
    try:
        s.set_shape(T, 0, 0, 0, arena)
        for c in meta:
            r = s.scan(models[c["model"]], arrays["dsq." + c["seq"]], c["i0"], c["j0"], algo=c["algo"], qdbidx=c["qdbidx"],
                       cutoff=c["cutoff"], do_null3=bool(c["null3"]), env_cutoff=c["env_cutoff"], want_vsc=True)
            _check(r.hits, r.envi, r.envj, r.sc, r.vsc, c, arrays)
    finally:
        s.close()
