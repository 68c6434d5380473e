"""The Infernal-side adapter against the reference's own scanners, on the CPU.

infernal_gb300/adapter/infernal_gb300_adapter.c defines Infernal's
FastCYKScan, FastIInsideScan, FastFInsideScan, RefTrCYKScan and
RefITrInsideScan with their exact prototypes (src/infernal.h:2710-2725) on
top of the C ABI.  oracle/build_ref.sh compiles it against the reference's
own headers; here it is linked with the reference's non-scanner objects
(cm_tophits.c, cm_mx.c, ...), the harness oracle/ref_harness.c (which builds
a CM_t and a scan matrix and calls the scanner symbols) and the
host-emulation build of the GPU library (the kernel source run on CPU
threads).  The same harness linked with the reference's own scanner objects
(oracle/_ref/libinfernal_ref.so) gives the reference's answer; every case
compares the CM_TOPHITS the call leaves behind (every hit, in order, with
every field a scanner sets: coordinates, root, mode, score, srcL, flags,
hit index, ...), the envelope, the best score, the per-state scores and the
truncation mode, bit for bit.
"""
import ctypes
import os
import subprocess
import zlib

import numpy as np
import pytest

import oracle
from infernal_gb300 import cmfile, emit

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_OBJ = os.path.join(ROOT, "oracle", "_ref", "obj")
ADAPTER_OBJ = os.path.join(ROOT, "oracle", "_ref", "adapter_obj")
NEXTRA = 12          # REFH_NEXTRA of ref_harness.c
P, I, I64, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float

pytestmark = pytest.mark.skipif(not (os.path.exists(oracle.REF_SO) and os.path.isdir(ADAPTER_OBJ)),
                                reason="reference scanners / adapter objects not built here (oracle/build_ref.sh)")


def _bind(path):
    lib = ctypes.CDLL(path)
    lib.refh_scan_full.argtypes = [P, I, I, I, P, I64, I64, F, I, F, I, I, P, I64, P, P, P, P, P, P, P, P]
    lib.refh_scan_full.restype = I
    return lib


@pytest.fixture(scope="module")
def libs(emu):
    """(reference harness library, adapter harness library)."""
    emu_so = os.path.join(ROOT, "tests", "emu", "_build", "libinfernal_gb300_emu.so")
    out = os.path.join(ROOT, "tests", "emu", "_build", "libadapter_test.so")
    objs = [os.path.join(ADAPTER_OBJ, f) for f in ("adapter.o", "adapter_stubs.o")]
    objs += [os.path.join(REF_OBJ, f + ".o") for f in ("ref_harness", "ref_offpath", "cm_mx", "cm_tophits", "cm_trunc",
                                                       "cm_qdband", "display", "cm_modelconfig", "logsum")]
    tmp = out + f".tmp{os.getpid()}"
    subprocess.check_call(["gcc", "-shared", "-o", tmp] + objs +
                          [emu_so, "-Wl,-rpath," + os.path.dirname(emu_so), "-Wl,-Bsymbolic", "-lm"])
    os.replace(tmp, out)
    return _bind(oracle.REF_SO), _bind(out)


def _run(lib, m, algo, qdbidx, dsq, i0, j0, cutoff, null3, env_cut, pass_idx, notgreedy, want_vsc=True):
    keep = []
    desc = cmfile.make_desc(m, flags_extra=(4 if notgreedy else 0), keep=keep)
    dsq = np.ascontiguousarray(dsq, np.uint8)
    nmax = 50000
    hits = (oracle._Hit * nmax)()
    extra = np.zeros(nmax * NEXTRA, np.int64)
    nh, ei, ej, sc, mode = I64(), I64(), I64(), F(), I()
    vsc = np.full(m.M, -1.0, np.float32)
    err = ctypes.create_string_buffer(256)
    st = lib.refh_scan_full(ctypes.byref(desc), m.nodes, oracle.REF_ALGOS[algo], qdbidx, dsq.ctypes.data, i0, j0, cutoff,
                            int(null3), env_cut, pass_idx, 1, ctypes.cast(hits, P), nmax, ctypes.byref(nh),
                            ctypes.byref(ei), ctypes.byref(ej), vsc.ctypes.data if want_vsc else None, ctypes.byref(sc),
                            ctypes.byref(mode), extra.ctypes.data, err)
    assert st == 0, err.value.decode()
    n = nh.value
    H = [(hits[k].start, hits[k].stop, hits[k].root, hits[k].mode, np.float32(hits[k].score).view(np.uint32)) for k in range(n)]
    X = [tuple(extra[k * NEXTRA:(k + 1) * NEXTRA]) for k in range(n)]
    return H, X, ei.value, ej.value, np.float32(sc.value).view(np.uint32), vsc.view(np.uint32), mode.value


def _target(m, rng, n, emitted=1):
    ins = [emit.sample(m, rng) for _ in range(emitted)]
    dsq, _ = emit.make_target(rng, n, 0.45, ins)
    return dsq


STD_CASES = [  # model, algo, band set, cutoff, NULL3, non-greedy, i0 offset
    ("tRNA", "cyk", 1, 0.0, True, False, 0), ("tRNA", "cyk", 0, 2.0, False, False, 37),
    ("tRNA", "inside", 2, 0.0, True, False, 0), ("tRNA", "finside", 2, 1.0, True, False, 0),
    ("tRNA", "cyk", 1, 0.0, True, True, 0), ("tRNA", "inside", 2, 0.0, False, True, 11),
    ("Vault", "cyk", 1, 0.0, True, False, 0), ("Vault", "inside", 2, 0.0, True, False, 5),
]


@pytest.mark.parametrize("name,algo,qdb,cut,null3,ng,off", STD_CASES)
def test_adapter_standard_scanners_equal_reference(libs, models, name, algo, qdb, cut, null3, ng, off):
    ref, ad = libs
    m = models[name]
    rng = np.random.default_rng(zlib.crc32(f"{name}{algo}{qdb}{ng}".encode()))
    dsq = _target(m, rng, 900, 2)
    L = len(dsq) - 2
    a = _run(ref, m, algo, qdb, dsq, 1 + off, L, cut, null3, 2.0, 0, ng)
    b = _run(ad, m, algo, qdb, dsq, 1 + off, L, cut, null3, 2.0, 0, ng)
    assert a[0], "the case should report hits"
    assert a[0] == b[0]                # hits in hit-list order: start, stop, root, mode, score bits
    assert a[1] == b[1]                # srcL, flags, hit index, ... of every hit
    assert a[2:5] == b[2:5]            # envelope, best score
    assert np.array_equal(a[5], b[5])  # per-state scores
    assert a[6] == b[6]


@pytest.mark.parametrize("algo,pass_idx,qdb,ng", [("trcyk", 2, 1, False), ("trcyk", 3, 1, False), ("trcyk", 4, 1, False),
                                                  ("trinside", 4, 2, False), ("trinside", 2, 0, True), ("trcyk", 3, 2, True)])
def test_adapter_truncated_scanners_equal_reference(libs, models, algo, pass_idx, qdb, ng):
    ref, ad = libs
    m = models["tRNA"]
    rng = np.random.default_rng(100 + pass_idx)
    e = emit.sample(m, rng)
    cut5, cut3 = len(e) // 3, 2 * len(e) // 3
    frag = {2: e[cut5:], 3: e[:cut3], 4: e[cut5:cut3]}[pass_idx]
    pad = "".join(rng.choice(list("ACGU"), 20))
    # a 5'-truncated hit starts at the read's first residue, a 3'-truncated one ends at its last
    seq = frag + pad if pass_idx == 2 else (pad + frag if pass_idx == 3 else frag)
    dsq = cmfile.digitize(seq)
    L = len(dsq) - 2
    a = _run(ref, m, algo, qdb, dsq, 1, L, -2.0, True, 1.0, pass_idx, ng)
    b = _run(ad, m, algo, qdb, dsq, 1, L, -2.0, True, 1.0, pass_idx, ng)
    assert a[0], "the case should report hits"
    assert a[0] == b[0]
    assert a[1] == b[1]
    assert a[2:5] == b[2:5]
    assert np.array_equal(a[5], b[5])
    assert a[6] == b[6]                # best truncation mode


def test_adapter_contract_errors(libs, models):
    """The reference's contract: an inverted range is eslEINCOMPAT with the
    reference's message; the reference-order scanners are not provided."""
    _, ad = libs
    m = models["tRNA"]
    keep = []
    desc = cmfile.make_desc(m, keep=keep)
    dsq = cmfile.digitize("ACGU" * 50)
    err = ctypes.create_string_buffer(256)
    nh, ei, ej, sc, mode = I64(), I64(), I64(), F(), I()
    hits = (oracle._Hit * 4)()
    st = ad.refh_scan_full(ctypes.byref(desc), m.nodes, oracle.REF_ALGOS["cyk"], 1, dsq.ctypes.data, 50, 10, 0.0, 1, 0.0, 0,
                           1, ctypes.cast(hits, P), 4, ctypes.byref(nh), ctypes.byref(ei), ctypes.byref(ej), None,
                           ctypes.byref(sc), ctypes.byref(mode), None, err)
    assert st == 10 and err.value.decode().startswith("FastCYKScan, i0: 50 j0: 10")
    st = ad.refh_scan_full(ctypes.byref(desc), m.nodes, oracle.REF_ALGOS["refinside"], 1, dsq.ctypes.data, 1, 100, 0.0, 1,
                           0.0, 0, 1, ctypes.cast(hits, P), 4, ctypes.byref(nh), ctypes.byref(ei), ctypes.byref(ej), None,
                           ctypes.byref(sc), ctypes.byref(mode), None, err)
    assert st == 10 and "not provided" in err.value.decode()
