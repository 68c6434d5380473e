"""Parity oracle for the GB300 scanners -- TEST INFRASTRUCTURE ONLY.

Two checkers live here:
  * the CPU restatement ``cm_scan_oracle.c`` (built on any machine into
    ``oracle/_build/liboracle.so``), and
  * the reference's own scanner sources compiled from the reference tree
    (``oracle/_ref/libinfernal_ref.so``, built by ``build_ref.sh`` where the
    reference tree exists), used to pin the restatement through golden vectors.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this package; the product (infernal_gb300/) never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
ORACLE_SO = os.path.join(BUILD, "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libinfernal_ref.so")

P, I, I64, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float
ALGOS = {"cyk": 0, "inside": 1, "finside": 2, "dinside": 3}
REF_ALGOS = {"cyk": 0, "refcyk": 1, "inside": 2, "refinside": 3, "finside": 4, "reffinside": 5,
             "trcyk": 6, "trinside": 7}


def build_oracle(force: bool = False) -> str:
    """Compiles the C restatement (gcc, no FMA contraction so that every float
    operation rounds as in the reference's C source)."""
    src = os.path.join(HERE, "cm_scan_oracle.c")
    if force or not os.path.exists(ORACLE_SO) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        os.makedirs(BUILD, exist_ok=True)
        tmp = ORACLE_SO + f".tmp{os.getpid()}"
        subprocess.check_call(["gcc", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-o", tmp, src, "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


REF_ROOT_ENV = "INFERNAL_REF_ROOT"      # where the reference tree is, in a container that has it


def reference_root() -> Optional[str]:
    """The reference tree's location: the INFERNAL_REF_ROOT environment variable."""
    return os.environ.get(REF_ROOT_ENV) or None


def build_ref(ref_root: Optional[str] = None) -> Optional[str]:
    """Builds oracle/_ref from the reference tree at ref_root (default: the
    INFERNAL_REF_ROOT environment variable) when that tree exists; returns
    the library path, or None without a tree."""
    ref_root = ref_root or reference_root()
    if not ref_root or not os.path.isdir(os.path.join(ref_root, "src")):
        return None
    subprocess.check_call([os.path.join(HERE, "build_ref.sh"), ref_root], stdout=subprocess.DEVNULL)
    return REF_SO


class _Hit(ctypes.Structure):
    _fields_ = [("start", I64), ("stop", I64), ("root", I), ("mode", I), ("score", F)]


_lib = {}


def _load(path):
    if path not in _lib:
        lib = ctypes.CDLL(path)
        if hasattr(lib, "oracle_scan"):
            lib.oracle_scan.argtypes = [P, I, I, P, I64, I64, F, I, F, I, P, I64, P, P, P, P, P, P]
            lib.oracle_scan.restype = I
        if hasattr(lib, "oracle_tr_scan"):
            lib.oracle_tr_scan.argtypes = [P, I, I, I, P, I64, I64, F, I, F, I, P, I64, P, P, P, P, P, P, P]
            lib.oracle_tr_scan.restype = I
        if hasattr(lib, "refh_tr_penalties"):
            lib.refh_tr_penalties.argtypes = [I, I, I] + [P] * 10 + [F] + [P] * 7
            lib.refh_tr_penalties.restype = I
        if hasattr(lib, "refh_qdb_bands"):
            lib.refh_qdb_bands.argtypes = [I, I, I] + [P] * 8 + [F, ctypes.c_double, ctypes.c_double,
                                                                 ctypes.c_double] + [P] * 6
            lib.refh_qdb_bands.restype = I
        if hasattr(lib, "refh_scan"):
            lib.refh_scan.argtypes = [P, I, I, I, P, I64, I64, F, I, F, I, I, P, I64, P, P, P, P, P, P, P]
            lib.refh_scan.restype = I
        _lib[path] = lib
    return _lib[path]


def scan(m, dsq, i0, j0, algo="cyk", qdbidx=1, cutoff=0.0, do_null3=True, env_cutoff=0.0,
         want_hits=True, notgreedy=False, reference=False, pass_idx=0, max_hits=200000):
    """Runs the restatement (reference=False) or the reference's own scanner
    (reference=True) and returns (hits, envi, envj, sc, vsc)."""
    from infernal_gb300 import cmfile
    keep: list = []
    desc = cmfile.make_desc(m, flags_extra=(4 if notgreedy else 0), keep=keep)
    dsq = np.ascontiguousarray(dsq, dtype=np.uint8)
    hits = (_Hit * max_hits)()
    nh, ei, ej, sc, mode = I64(), I64(), I64(), F(), I()
    vsc = np.zeros(m.M, np.float32)
    err = ctypes.create_string_buffer(256)
    if reference:
        lib = _load(REF_SO)
        st = lib.refh_scan(ctypes.byref(desc), m.nodes, REF_ALGOS[algo], qdbidx, dsq.ctypes.data, i0, j0,
                           cutoff, int(do_null3), env_cutoff, pass_idx, int(want_hits), ctypes.cast(hits, P),
                           max_hits, ctypes.byref(nh), ctypes.byref(ei), ctypes.byref(ej), vsc.ctypes.data,
                           ctypes.byref(sc), ctypes.byref(mode), err)
    else:
        lib = _load(build_oracle())
        st = lib.oracle_scan(ctypes.byref(desc), ALGOS[algo], qdbidx, dsq.ctypes.data, i0, j0, cutoff,
                             int(do_null3), env_cutoff, int(want_hits), ctypes.cast(hits, P), max_hits,
                             ctypes.byref(nh), ctypes.byref(ei), ctypes.byref(ej), vsc.ctypes.data,
                             ctypes.byref(sc), err)
    if st != 0:
        raise RuntimeError(f"oracle status {st}: {err.value.decode()}")
    H = [(hits[k].start, hits[k].stop, hits[k].root, hits[k].mode, hits[k].score) for k in range(min(nh.value, max_hits))]
    return H, ei.value, ej.value, sc.value, vsc


TR_ALGOS = {"trcyk": 0, "trinside": 1}


def tr_scan(m, dsq, i0, j0, algo="trcyk", qdbidx=1, pass_idx=4, cutoff=0.0, do_null3=True, env_cutoff=0.0,
            want_hits=True, notgreedy=False, reference=False, max_hits=200000):
    """Truncated scan (RefTrCYKScan / RefITrInsideScan) by the restatement or
    the reference; returns (hits, envi, envj, sc, vsc, mode)."""
    from infernal_gb300 import cmfile
    keep: list = []
    desc = cmfile.make_desc(m, flags_extra=(4 if notgreedy else 0), keep=keep)
    dsq = np.ascontiguousarray(dsq, dtype=np.uint8)
    hits = (_Hit * max_hits)()
    nh, ei, ej, sc, mode = I64(), I64(), I64(), F(), I()
    vsc = np.zeros(m.M, np.float32)
    err = ctypes.create_string_buffer(256)
    if reference:
        lib = _load(REF_SO)
        st = lib.refh_scan(ctypes.byref(desc), m.nodes, REF_ALGOS[algo], qdbidx, dsq.ctypes.data, i0, j0,
                           cutoff, int(do_null3), env_cutoff, pass_idx, int(want_hits), ctypes.cast(hits, P),
                           max_hits, ctypes.byref(nh), ctypes.byref(ei), ctypes.byref(ej), vsc.ctypes.data,
                           ctypes.byref(sc), ctypes.byref(mode), err)
    else:
        lib = _load(build_oracle())
        st = lib.oracle_tr_scan(ctypes.byref(desc), TR_ALGOS[algo], qdbidx, pass_idx, dsq.ctypes.data, i0, j0,
                                cutoff, int(do_null3), env_cutoff, int(want_hits), ctypes.cast(hits, P), max_hits,
                                ctypes.byref(nh), ctypes.byref(ei), ctypes.byref(ej), vsc.ctypes.data,
                                ctypes.byref(sc), ctypes.byref(mode), err)
    if st != 0:
        raise RuntimeError(f"oracle status {st}: {err.value.decode()}")
    H = [(hits[k].start, hits[k].stop, hits[k].root, hits[k].mode, hits[k].score) for k in range(min(nh.value, max_hits))]
    return H, ei.value, ej.value, sc.value, vsc, mode.value


def ref_tr_penalties(m):
    """Truncation penalties and emit map computed by the reference's own
    cm_tr_penalties_Create / CreateEmitMap (oracle/_ref); returns
    (lpos, rpos, g, l, ig, il) with the penalty tables shaped [3, M]."""
    lib = _load(REF_SO)
    M, n = m.M, m.nodes
    keep = []

    def c(a, dt):
        x = np.ascontiguousarray(a, dt)
        keep.append(x)
        return x.ctypes.data
    lp, rp = np.zeros(n, np.int32), np.zeros(n, np.int32)
    g, l = np.zeros(3 * M, np.float32), np.zeros(3 * M, np.float32)
    ig, il = np.zeros(3 * M, np.int32), np.zeros(3 * M, np.int32)
    err = ctypes.create_string_buffer(256)
    st = lib.refh_tr_penalties(M, n, m.clen, c(m.sttype, np.int8), c(m.stid, np.int8), c(m.ndidx, np.int32),
                               c(m.cfirst, np.int32), c(m.cnum, np.int32), c(m.plast, np.int32),
                               c(m.pnum, np.int32), c(m.ndtype, np.int8), c(m.nodemap, np.int32),
                               c(m.t_global, np.float32), float(m.pbegin), lp.ctypes.data, rp.ctypes.data,
                               g.ctypes.data, l.ctypes.data, ig.ctypes.data, il.ctypes.data, err)
    if st != 0:
        raise RuntimeError(f"refh_tr_penalties status {st}: {err.value.decode()}")
    return lp, rp, g.reshape(3, M), l.reshape(3, M), ig.reshape(3, M), il.reshape(3, M)


def ref_qdb_bands(m, beta1=1e-7, beta2=1e-15, beta_W=1e-7):
    """Bands and W by the reference's own CalculateQueryDependentBands
    (oracle/_ref); returns (dmin1, dmax1, dmin2, dmax2, W)."""
    lib = _load(REF_SO)
    keep = []

    def c(a, dt):
        x = np.ascontiguousarray(a, dt)
        keep.append(x)
        return x.ctypes.data
    out = [np.zeros(m.M, np.int32) for _ in range(4)]
    W = I()
    err = ctypes.create_string_buffer(256)
    st = lib.refh_qdb_bands(m.M, m.nodes, m.clen, c(m.sttype, np.int8), c(m.stid, np.int8), c(m.cfirst, np.int32),
                            c(m.cnum, np.int32), c(m.pnum, np.int32), c(m.ndtype, np.int8), c(m.nodemap, np.int32),
                            c(m.t_global, np.float32), float(m.pbegin), beta1, beta2, beta_W,
                            *[o.ctypes.data for o in out], ctypes.byref(W), err)
    if st != 0:
        raise RuntimeError(f"refh_qdb_bands status {st}: {err.value.decode()}")
    return out[0], out[1], out[2], out[3], W.value
