"""Inside against a double-precision yardstick: the FastFInsideScan recursion
in double with the exact log-sum and IMPOSSIBLE as -infinity
(oracle/cm_scan_oracle.c core_dinside).  The table-based Inside scanners
(integer ILogsum, float FLogsum) are the reference's own arithmetic, so their
distance from FP64 is the reference's table error; it is stated here per
model.  The GPU scanners reproduce the table-based scores bit for bit
(tests/test_gpu_parity.py), so these bounds hold for them too; the GPU leg
below checks that directly on the device."""
import numpy as np
import pytest

import oracle
from infernal_gb300 import cmfile, emit, lib as L


def _case(m, name, seed):
    rng = np.random.default_rng(seed)
    ins = [emit.sample(m, rng)]
    n = 900 if name == "Plant_SRP" else 1500
    dsq, _ = emit.make_target(rng, n, 0.45, ins)
    return dsq


def _errors(hits, ref):
    d = {(h[0], h[1]): h[4] for h in ref}
    e = [abs(h[4] - d[(h[0], h[1])]) for h in hits if (h[0], h[1]) in d]
    return e


@pytest.mark.parametrize("name", ["tRNA", "Vault", "Plant_SRP"])
def test_table_inside_error_vs_fp64(models, name):
    m = models[name]
    dsq = _case(m, name, 3)
    n = len(dsq) - 2
    ref = oracle.scan(m, dsq, 1, n, algo="dinside", qdbidx=2, cutoff=0.0, env_cutoff=5.0)
    for algo, bound in (("inside", 0.1), ("finside", 0.01)):
        r = oracle.scan(m, dsq, 1, n, algo=algo, qdbidx=2, cutoff=0.0, env_cutoff=5.0)
        e = _errors(r[0], ref[0])
        assert len(e) >= 1
        assert max(e) < bound and abs(r[3] - ref[3]) < bound


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["tRNA", "Vault", "Plant_SRP"])
def test_gpu_inside_error_vs_fp64(models, name):
    m = models[name]
    dsq = _case(m, name, 5)      # seed 5: the FP64 scan reports at least one hit for every model
    n = len(dsq) - 2
    ref = oracle.scan(m, dsq, 1, n, algo="dinside", qdbidx=2, cutoff=0.0, env_cutoff=5.0)
    assert len(ref[0]) >= 1
    s = L.Scanner(0)
    try:
        for algo, bound in (("inside", 0.1), ("finside", 0.01)):
            r = s.scan(m, dsq, 1, n, algo=algo, qdbidx=2, cutoff=0.0, env_cutoff=5.0)
            e = _errors(r.hits, ref[0])
            print(f"{name} {algo}: {len(e)} hits, max |GPU - FP64| {max(e):.4f} bits, mean {np.mean(e):.4f}, "
                  f"best score {abs(r.sc - ref[3]):.4f}")
            assert len(e) >= 1 and max(e) < bound
    finally:
        s.close()
