"""E-value calibration (cmgb_Calibrate): the exponential tail fitted on the
GPU to the best hits of 1.6 Mb of seeded random sequence, against the
calibration stored in the reference's CM files (ECMLC / ECMLI lines of
testsuite/*.c.cm, written by the reference's cmcalibrate).  The random
backgrounds differ (the reference samples a genomic HMM; this one uses
GC-varying iid segments), so the comparison is statistical: the E = 0.01
score threshold of a 1 Mb search and lambda agree within stated bounds."""
import ctypes

import numpy as np
import pytest

from infernal_gb300 import lib as L


def test_evalue_formula_matches_the_reference_fields(models):
    # E = Z / dbsize * nrandhits * exp(-lambda (S - mu_extrap)); ECMLI of Plant_SRP.c.cm
    ecm = models["Plant_SRP"].ecm["ECMLI"]
    assert ecm == (0.70748, -9.17856, -0.59906, 1600000.0, 519142.0, 0.002312)
    s = L.bits_at_evalue(ecm, 0.01, 4e6)
    assert abs(L.evalue(ecm, s, 4e6) - 0.01) < 1e-9
    assert 17.0 < s < 17.4
    # mu_extrap = mu_orig - log(1 / tailp) / lambda, as cmcalibrate stores it
    lam, mu_x, mu_o, _, _, tailp = ecm
    assert abs(mu_o - np.log(1.0 / tailp) / lam - mu_x) < 1e-3
    # the tail-only form (nrandhits = tail size, tailp = 1) gives the same E-values
    tail = (lam, mu_o, mu_o, ecm[3], ecm[4] * tailp, 1.0)
    assert abs(L.bits_at_evalue(tail, 0.01, 4e6) - s) < 0.01


def test_expinfo_layout():
    assert ctypes.sizeof(L.ExpInfo) == 48


@pytest.mark.gpu
@pytest.mark.parametrize("name,algo,tag", [("Vault", "cyk", "ECMLC"), ("Vault", "inside", "ECMLI"),
                                           ("Plant_SRP", "cyk", "ECMLC"), ("Plant_SRP", "inside", "ECMLI")])
def test_gpu_calibration_matches_cm_file(models, name, algo, tag):
    m = models[name]
    s = L.Scanner(0)
    try:
        ours, ms = s.calibrate(m, algo=algo, total_len=1_600_000, seq_len=100_000, seed=181, tail_per_mb=750)
    finally:
        s.close()
    ref = m.ecm[tag]
    b_ours, b_ref = L.bits_at_evalue(ours, 0.01, 1e6), L.bits_at_evalue(ref, 0.01, 1e6)
    print(f"{name} {tag}: lambda {ours[0]:.4f} (file {ref[0]:.4f}), mu {ours[2]:.3f} (file {ref[2]:.3f}), "
          f"E=0.01 @ 1 Mb: {b_ours:.2f} bits (file {b_ref:.2f}); {ms:.0f} ms of scanning")
    assert ours[4] == 1200 and ours[5] == 1.0 and ours[3] == 1.6e6
    # measured on a GB300: tail origin within 0.05 bits, lambda within 0.06,
    # the E = 0.01 threshold within 1.5 bits of the file's calibration
    assert abs(ours[2] - ref[2]) < 0.5
    assert abs(ours[0] - ref[0]) < 0.1
    assert abs(b_ours - b_ref) < 2.0


@pytest.mark.gpu
@pytest.mark.parametrize("name,algo,tag", [("Vault", "cyk", "ECMGC"), ("Vault", "inside", "ECMGI"),
                                           ("tRNA", "cyk", "ECMGC")])
def test_gpu_glocal_calibration(name, algo, tag):
    """Glocal modes: the model configured without local begins or ends, the
    tail of 250 hits per Mb (the reference's --gtailn)."""
    import os
    from infernal_gb300 import cmfile
    m = cmfile.load_npz(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", f"{name}.glocal.model.npz"))
    s = L.Scanner(0)
    try:
        ours, ms = s.calibrate(m, algo=algo, total_len=1_600_000, seq_len=100_000, seed=181, tail_per_mb=250)
    finally:
        s.close()
    ref = m.ecm[tag]
    b_ours, b_ref = L.bits_at_evalue(ours, 0.01, 1e6), L.bits_at_evalue(ref, 0.01, 1e6)
    print(f"{name} {tag}: lambda {ours[0]:.4f} (file {ref[0]:.4f}), mu {ours[2]:.3f} (file {ref[2]:.3f}), "
          f"E=0.01 @ 1 Mb: {b_ours:.2f} bits (file {b_ref:.2f}); {ms:.0f} ms of scanning")
    assert ours[4] == 400 and ours[5] == 1.0
    assert abs(ours[2] - ref[2]) < 3.0
    assert abs(ours[0] - ref[0]) < 0.25 * ref[0]
    assert abs(b_ours - b_ref) < 4.0
