"""The CYK kernels take maxima with the max instruction, which equals the
reference's ESL_MAX(a, b) = a > b ? a : b bit for bit unless a and b are zeros
of opposite sign.  A DP value is -0.0 only if a score table entry is -0.0
(IEEE addition gives -0.0 only for -0.0 + -0.0); the configured models'
tables hold none, and cmgb_model_create stores any -0.0 entry as +0.0."""
import glob
import os

import numpy as np
import pytest

from infernal_gb300 import cmfile

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MODELS = sorted(glob.glob(os.path.join(GOLDEN, "*.model.npz")) + glob.glob(os.path.join(GOLDEN, "panel", "*.model.npz")))


def _neg_zero(a):
    a = np.asarray(a, np.float32).ravel()
    return int(np.count_nonzero((a == 0) & np.signbit(a)))


@pytest.mark.parametrize("path", MODELS, ids=[os.path.basename(p) for p in MODELS])
def test_configured_tables_hold_no_negative_zero(path):
    m = cmfile.load_npz(path)
    for tab in ("tsc", "oesc", "endsc", "beginsc", "lmesc", "rmesc", "tr_g_pty", "tr_l_pty"):
        a = getattr(m, tab, None)
        if a is not None:
            assert _neg_zero(a) == 0, tab
    assert not (m.el_selfsc == 0 and np.signbit(np.float32(m.el_selfsc)))

