"""The allocation-free CYK entry point, through the C ABI.

cmgb_FastCYKScan_noalloc is for callers that cannot call cudaMalloc while
they scan: a host program whose own allocator (a framework's caching
allocator, a pool sized at start-up) owns the device memory, and
long-running services that allocate only at start-up because cudaMalloc can
fail under load and synchronises the whole device.  Its scratch is a static
device array shared by every call; its outputs go to caller-provided device
memory.  This test checks it against the existing device-resident entry
point (cmgb_FastCYKScan_dev) on the same inputs, on two calls in a row (the
static array keeps the previous call's contents), bit for bit as the other
CYK parity tests do: same envelope, same best score, and every hit that entry
point reports is one of the returned cells with the same score and root.
Greedy models return the cells at or above the cutoff; a model flagged
non-greedy returns every cell above zero, the candidates of optimal
resolution.  It lives in its own file, collected last."""
import ctypes

import numpy as np
import pytest

from infernal_gb300 import emit, lib as L

pytestmark = pytest.mark.gpu

CELL = np.dtype([("j", np.int64), ("d", np.int32), ("score", np.float32), ("root", np.int32), ("pad", np.int32)])


@pytest.mark.parametrize("name,notgreedy", [("tRNA", False), ("Vault", False), ("tRNA", True)])
def test_no_alloc_matches_device_entry_point(models, name, notgreedy):
    torch = pytest.importorskip("torch")
    m = models[name]
    rng = np.random.default_rng(77)
    inserts = [emit.sample(m, rng) for _ in range(6)]
    dsq, _ = emit.make_target(rng, 60000 if not notgreedy else 20000, 0.45, inserts)
    n = len(dsq) - 2
    d_dsq = torch.from_numpy(dsq).cuda()
    cap = 1 << 20
    d_cells = torch.zeros(cap * CELL.itemsize, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    sc = L.Scanner(0)
    try:
        cutoff = 3.0
        # the existing entry point (also builds the model's plan for band set 1)
        ref = sc.scan(m, None, 1, n, algo="cyk", qdbidx=1, cutoff=cutoff, do_null3=False, env_cutoff=2.0,
                      notgreedy=notgreedy, device_ptr=d_dsq.data_ptr())
        mh = sc.model(m, L.CMGB_NOTGREEDY if notgreedy else 0)
        for call in range(2):
            ncells, envi, envj, best = ctypes.c_int(), ctypes.c_int64(), ctypes.c_int64(), ctypes.c_float()
            err = ctypes.create_string_buffer(256)
            st = sc.lib.cmgb_FastCYKScan_noalloc(sc._ctx, mh, err, 1, d_dsq.data_ptr(), 1, n, cutoff, 2.0,
                                                  d_cells.data_ptr(), cap, ctypes.byref(ncells), ctypes.byref(envi),
                                                  ctypes.byref(envj), ctypes.byref(best))
            assert st == 0, err.value
            assert (envi.value, envj.value) == (ref.envi, ref.envj)
            assert np.float32(best.value) == np.float32(ref.sc)
            cells = np.frombuffer(d_cells[: ncells.value * CELL.itemsize].cpu().numpy().tobytes(), dtype=CELL)
            assert len(cells) == ncells.value > 0
            if notgreedy:
                assert (cells["score"] > 0).all()
            else:
                assert (cells["score"] >= cutoff).all()
            assert cells["score"].max() == np.float32(ref.sc)
            # every hit of the existing entry point (no NULL3) is one of the cells, with the same score and root
            table = {(int(c["j"]), int(c["d"])): (float(c["score"]), int(c["root"])) for c in cells}
            assert len(table) == len(cells)
            assert ref.hits
            for (start, stop, root, mode, score) in ref.hits:
                assert table[(stop, stop - start + 1)] == (score, root)
    finally:
        sc.close()
