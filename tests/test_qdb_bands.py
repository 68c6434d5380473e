"""Query-dependent band calculation (cmfile.qdb_bands, the host restatement
of CalculateQueryDependentBands / BandCalculationEngine, src/cm_qdband.c)
against the reference's own compiled engine, at the default betas and at
others; and W against the value stored in the CM files."""
import os

import numpy as np
import pytest

import oracle
from infernal_gb300 import cmfile


def test_w_matches_cm_files(models):
    for m in models.values():
        assert cmfile.qdb_bands(m)[4] == m.W


def test_bands_close_to_cm_files(models):
    """The files' bands were computed by cmbuild from unrounded parameters;
    recomputed from the file's rounded ones they stay within one residue."""
    for m in models.values():
        for a, b in zip(cmfile.qdb_bands(m)[:4], (m.dmin1, m.dmax1, m.dmin2, m.dmax2)):
            assert np.abs(a.astype(int) - b.astype(int)).max() <= 1


@pytest.mark.skipif(not os.path.exists(oracle.REF_SO), reason="reference library not built here")
@pytest.mark.parametrize("betas", [(1e-7, 1e-15, 1e-7), (1e-5, 1e-9, 1e-6), (1e-3, 1e-4, 1e-3)])
def test_bands_equal_reference(models, betas):
    for m in models.values():
        mine = cmfile.qdb_bands(m, *betas)
        ref = oracle.ref_qdb_bands(m, *betas)
        assert mine[4] == ref[4]
        for a, b in zip(mine[:4], ref[:4]):
            assert np.array_equal(a, b)


def test_beta_order_enforced(models):
    with pytest.raises(ValueError):
        cmfile.qdb_bands(models["tRNA"], 1e-15, 1e-7)
