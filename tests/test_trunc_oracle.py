"""Truncated scanning on the CPU: the truncation tables of the host model layer
and the restatement of RefTrCYKScan / RefITrInsideScan against the golden
vectors written by the reference's own truncated scanners
(tests/golden/gen_golden.py)."""
import os

import numpy as np
import pytest

import oracle
from conftest import hits_from_golden
from infernal_gb300 import cmfile

TR = ("trcyk", "trinside")


def _tr_cases(golden):
    meta, _ = golden
    return [c for c in meta if c["algo"] in TR]


def test_truncated_cases_present(golden):
    cases = _tr_cases(golden)
    assert len(cases) >= 60
    assert {c["pass_idx"] for c in cases} == {2, 3, 4, 5}
    assert {c["mode"] for c in cases} >= {1, 2, 3}            # R, L and J best parses
    assert sum(1 for c in cases if c["hits"]) >= 30
    assert any(c["notgreedy"] for c in cases) and any(c["qdbidx"] == 0 for c in cases)


@pytest.mark.parametrize("idx", range(0, 70))
def test_tr_oracle_matches_reference(golden, models, idx):
    cases = _tr_cases(golden)
    if idx >= len(cases):
        pytest.skip("no such case")
    c = cases[idx]
    _, arrays = golden
    m = models[c["model"]]
    dsq = arrays["dsq." + c["seq"]]
    hits, ei, ej, sc, vsc, mode = oracle.tr_scan(m, dsq, c["i0"], c["j0"], algo=c["algo"], qdbidx=c["qdbidx"],
                                                 pass_idx=c["pass_idx"], cutoff=c["cutoff"],
                                                 do_null3=bool(c["null3"]), env_cutoff=c["env_cutoff"],
                                                 notgreedy=bool(c["notgreedy"]))
    assert hits == hits_from_golden(c)
    assert (ei, ej) == (c["envi"], c["envj"])
    assert np.float32(sc) == np.float32(float.fromhex(c["sc"]))
    assert mode == c["mode"]
    assert np.array_equal(vsc.view(np.int32), arrays[f"vsc.{c['id']}"].view(np.int32))


def test_tr_oracle_rejects_bad_pass(models):
    m = models["tRNA"]
    dsq = cmfile.digitize("ACGUACGUAC")
    for bad in (0, 1, 6):   # cm_TrFillFromPassIdx's eslEINVAL
        with pytest.raises(RuntimeError, match="status 11"):
            oracle.tr_scan(m, dsq, 1, 10, pass_idx=bad)


def test_emit_map_covers_consensus(models):
    for m in models.values():
        assert m.emap_rpos[0] - 1 == m.clen
        assert (m.emap_lpos >= 0).all() and (m.emap_lpos <= m.emap_rpos).all()


def test_penalty_tables_shape(models):
    for m in models.values():
        for a in (m.tr_g_pty, m.tr_l_pty, m.tr_ig_pty, m.tr_il_pty):
            assert a.shape == (3, m.M)
        # every state with a local penalty in one table has one in all three
        fin = m.tr_il_pty != -cmfile.INFTY
        assert (fin[0] == fin[1]).all() and (fin[0] == fin[2]).all()
        # truncated begins never enter BEGL_S, E or the root
        assert not fin[0][(m.stid == cmfile.BEGL_S) | (m.sttype == cmfile.E_st)].any()
        assert not fin[0][0]


@pytest.mark.skipif(not os.path.exists(oracle.REF_SO), reason="reference library not built here")
def test_penalties_equal_reference(models):
    """Pin: the host restatement of cm_tr_penalties_Create and CreateEmitMap
    reproduces the reference's own compiled functions bit for bit."""
    for m in models.values():
        lp, rp, g, l, ig, il = oracle.ref_tr_penalties(m)
        assert np.array_equal(lp, m.emap_lpos) and np.array_equal(rp, m.emap_rpos)
        assert np.array_equal(g.view(np.int32), m.tr_g_pty.view(np.int32))
        assert np.array_equal(l.view(np.int32), m.tr_l_pty.view(np.int32))
        assert np.array_equal(ig, m.tr_ig_pty) and np.array_equal(il, m.tr_il_pty)
