"""CPU tests of the C ABI: the built library exports every declared symbol,
and the kernel source -- compiled for the test-only host-thread emulation of a
CTA -- reproduces the oracle bit for bit and keeps the reference's error
behaviour.  No GPU is used."""
import os
import re

import numpy as np
import pytest

import oracle
from infernal_gb300 import cmfile, lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            src = open(os.path.join(ROOT, "include", fn)).read()
            src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
            names |= set(re.findall(r"\b(cmgb_\w+)\s*\(", src))
    return names


def test_header_and_binding_agree():
    assert _declared_functions() == set(L.EXPORTS)


def test_header_compiles_as_c_and_cpp(tmp_path):
    """The C ABI header stands alone: pedantic C99 (Infernal's C) and C++."""
    import subprocess
    for ext, cmd in (("c", ["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror"]),
                     ("cpp", ["g++", "-std=c++11", "-Wall", "-Wextra", "-Werror"])):
        src = tmp_path / f"h.{ext}"
        src.write_text('#include "infernal_gb300.h"\nint main(void) { return 0; }\n')
        subprocess.check_call(cmd + ["-fsyntax-only", "-I", os.path.join(ROOT, "include"), str(src)])


@pytest.fixture(scope="module")
def built_lib():
    import __graft_entry__ as g
    csrc = os.path.join(ROOT, "infernal_gb300", "csrc")
    newest = max(os.path.getmtime(os.path.join(csrc, f)) for f in os.listdir(csrc))
    newest = max(newest, os.path.getmtime(os.path.join(ROOT, "include", "infernal_gb300.h")))
    if not os.path.exists(L.LIB_PATH) or os.path.getmtime(L.LIB_PATH) < newest:
        g.build_library()
    return L.LIB_PATH


def test_library_exports_every_declared_symbol(built_lib):
    import ctypes
    lib = ctypes.CDLL(built_lib)      # loading touches no GPU
    for name in _declared_functions():
        assert hasattr(lib, name), name


def test_count_cells_matches_oracle(built_lib, models):
    import ctypes
    lib = L.bind(built_lib)
    olib = ctypes.CDLL(oracle.build_oracle())
    olib.oracle_count_cells.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int64]
    olib.oracle_count_cells.restype = ctypes.c_int64
    for m in models.values():
        keep = []
        d = cmfile.make_desc(m, keep=keep)
        for q in (0, 1, 2):
            for Ln in (10, m.W - 1, m.W, 5000):
                assert lib.cmgb_count_cells(ctypes.byref(d), q, Ln) == olib.oracle_count_cells(ctypes.byref(d), q, Ln)


@pytest.mark.parametrize("name,algo,qdb,T,win,arena", [
    ("tRNA", "cyk", 1, 4, 0, 1), ("tRNA", "inside", 2, 8, 0, 1), ("Vault", "cyk", 2, 16, 300, 1),
    ("tRNA", "cyk", 0, 16, 0, 2), ("Plant_SRP", "inside", 1, 40, 0, 2), ("Vault", "inside", 2, 64, 250, 2),
    ("tRNA", "finside", 2, 12, 0, 1)])
def test_emulated_kernel_matches_oracle(emu, models, name, algo, qdb, T, win, arena):
    m = models[name]
    rng = np.random.default_rng(11)
    n = 220 if name == "Plant_SRP" else 350
    dsq = cmfile.digitize("".join(rng.choice(list("ACGU"), n)))
    emu.set_shape(T, win, 1, 0, arena)
    r = emu.scan(m, dsq, 1, n, algo=algo, qdbidx=qdb, cutoff=-2.0, env_cutoff=1.0, want_vsc=True)
    o = oracle.scan(m, dsq, 1, n, algo=algo, qdbidx=qdb, cutoff=-2.0, env_cutoff=1.0)
    assert r.hits == o[0]
    assert (r.envi, r.envj) == (o[1], o[2]) and np.float32(r.sc) == np.float32(o[3])
    assert np.array_equal(r.vsc.view(np.int32), o[4].view(np.int32))


def test_emulated_golden_degenerate_case(emu, models, golden):
    """A golden case with degenerate residues and NULL3 through the emulated kernel."""
    from conftest import hits_from_golden
    meta, arrays = golden
    c = next(c for c in meta if c["seq"] == "tRNA.degen" and c["algo"] == "inside")
    emu.set_shape(8, 0, 1)
    r = emu.scan(models["tRNA"], arrays["dsq." + c["seq"]], c["i0"], c["j0"], algo="inside", qdbidx=c["qdbidx"],
                 cutoff=c["cutoff"], do_null3=bool(c["null3"]), env_cutoff=c["env_cutoff"])
    assert r.hits == hits_from_golden(c)


def test_contract_errors(emu, models):
    """eslEINCOMPAT on contract violations, as src/cm_dpsearch.c:129-154."""
    m = models["tRNA"]
    dsq = cmfile.digitize("ACGU" * 30)
    with pytest.raises(L.ScanError) as e:
        emu.scan(m, dsq, 50, 10)
    assert e.value.status == 10 and "i0" in str(e.value)
    with pytest.raises(L.ScanError) as e:
        emu.scan(m, dsq, 1, 100, qdbidx=3)
    assert e.value.status == 10
    with pytest.raises(L.ScanError) as e:
        emu.set_shape(-1, 0, 0)
    assert e.value.status == 11


def test_emulated_batch_with_many_candidates_matches_oracle(emu, models):
    """A batch whose candidate cells (every finite root cell at a very low
    cutoff, about 200,000 of them) are spread over the sequences by several
    host threads: every sequence's hits, envelope and best score equal the
    oracle's scan of that sequence."""
    m = models["tRNA"]
    rng = np.random.default_rng(17)
    seqs = [cmfile.digitize("".join(rng.choice(list("ACGU"), int(n)))) for n in rng.integers(150, 400, size=5)]
    emu.set_shape(16, 0, 1, 0, 2)
    try:
        rs = emu.scan_batch(m, seqs, algo="cyk", qdbidx=1, cutoff=-40.0, env_cutoff=1.0)
    finally:
        emu.set_shape(0, 0, 0)
    assert sum(len(s) - 2 for s in seqs) * 100 > 131072   # enough root cells for more than one slice
    for dsq, r in zip(seqs, rs):
        o = oracle.scan(m, dsq, 1, len(dsq) - 2, algo="cyk", qdbidx=1, cutoff=-40.0, env_cutoff=1.0)
        assert r.hits == o[0]
        assert (r.envi, r.envj) == (o[1], o[2]) and np.float32(r.sc) == np.float32(o[3])
