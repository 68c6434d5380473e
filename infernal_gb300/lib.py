"""ctypes bindings of the C ABI in include/infernal_gb300.h.

This is the Python mirror of the reference scanner interface
(``FastCYKScan``/``FastIInsideScan``, src/cm_dpsearch.c:90 and :1106;
``RefTrCYKScan``/``RefITrInsideScan``, src/cm_dpsearch_trunc.c:79 and :741): the
same argument meaning and the same error behaviour (a non-zero Easel status
code is raised as :class:`ScanError` carrying the errbuf text).

The shared library is the in-tree build ``infernal_gb300/_lib/libinfernal_gb300.so``
(``python -c "import __graft_entry__ as g; g.build()"``).  There is no CPU
fallback: if the library or a GPU is missing, :func:`load` raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass
from typing import List, Optional

import numpy as np

from . import cmfile

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libinfernal_gb300.so")

P, I, I64, F = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_float
CMGB_NOTGREEDY = 1 << 2

# every symbol the header declares (checked by the CPU tests)
EXPORTS = [
    "cmgb_logsum_init", "cmgb_ctx_create", "cmgb_ctx_destroy", "cmgb_ctx_set_shape",
    "cmgb_ctx_last_kernel_ms", "cmgb_ctx_last_launches", "cmgb_ctx_last_transfer_bytes", "cmgb_model_create", "cmgb_model_destroy",
    "cmgb_hitlist_create", "cmgb_hitlist_destroy", "cmgb_hitlist_count", "cmgb_hitlist_get",
    "cmgb_hitlist_clear", "cmgb_FastCYKScan", "cmgb_FastIInsideScan", "cmgb_FastCYKScan_dev",
    "cmgb_FastIInsideScan_dev", "cmgb_count_cells", "cmgb_autotune", "cmgb_FastCYKScan_noalloc",
    "cmgb_FastFInsideScan", "cmgb_FastFInsideScan_dev",
    "cmgb_RefTrCYKScan", "cmgb_RefITrInsideScan", "cmgb_RefTrCYKScan_dev", "cmgb_RefITrInsideScan_dev",
    "cmgb_ScanBatch", "cmgb_ScanMulti", "cmgb_Calibrate", "cmgb_filter_trainer_create", "cmgb_filter_trainer_destroy",
    "cmgb_filter_trainer_set", "cmgb_filter_trainer_step", "cmgb_filter_trainer_get", "cmgb_filter_create", "cmgb_filter_destroy", "cmgb_filter_windows",
    "cmgb_measure_issue_peak", "cmgb_ScanBatch_dev", "cmgb_filter_create_heads", "cmgb_filter_trainer_create_heads",
    "cmgb_filter_trainer_step_heads", "cmgb_ScanMulti_dev",
]
BATCH_ALGOS = {"cyk": 0, "inside": 1, "finside": 2, "trcyk": 3, "trinside": 4}

_SCAN_ARGS = [P, P, ctypes.c_char_p, I, P, I64, I64, F, P, I, F, P, P, P, P]
_TR_SCAN_ARGS = [P, P, ctypes.c_char_p, I, I, P, I64, I64, F, P, I, F, P, P, P, P, P]
TR_ALGOS = {"trcyk": "cmgb_RefTrCYKScan", "trinside": "cmgb_RefITrInsideScan"}


class Hit(ctypes.Structure):
    _fields_ = [("start", I64), ("stop", I64), ("root", I), ("mode", I), ("score", F)]


class ScanError(RuntimeError):
    """A scanner returned a non-zero status; .status is the Easel code."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"status {status}: {msg}")
        self.status = status


_libs = {}


def bind(path: str) -> ctypes.CDLL:
    """Loads a library exporting the C ABI and declares its prototypes."""
    if path in _libs:
        return _libs[path]
    lib = ctypes.CDLL(path)
    lib.cmgb_logsum_init.argtypes = []
    lib.cmgb_ctx_create.argtypes = [I, ctypes.POINTER(P), ctypes.c_char_p]
    lib.cmgb_ctx_create.restype = I
    lib.cmgb_ctx_destroy.argtypes = [P]
    lib.cmgb_ctx_set_shape.argtypes = [P, I, I, I, I, I]
    lib.cmgb_ctx_set_shape.restype = I
    lib.cmgb_ctx_last_kernel_ms.argtypes = [P]
    lib.cmgb_ctx_last_kernel_ms.restype = F
    lib.cmgb_ctx_last_launches.argtypes = [P]
    lib.cmgb_ctx_last_launches.restype = I
    lib.cmgb_ctx_last_transfer_bytes.argtypes = [P, ctypes.POINTER(I64), ctypes.POINTER(I64)]
    lib.cmgb_model_create.argtypes = [P, P, ctypes.POINTER(P), ctypes.c_char_p]
    lib.cmgb_model_create.restype = I
    lib.cmgb_model_destroy.argtypes = [P]
    lib.cmgb_hitlist_create.argtypes = []
    lib.cmgb_hitlist_create.restype = P
    lib.cmgb_hitlist_destroy.argtypes = [P]
    lib.cmgb_hitlist_count.argtypes = [P]
    lib.cmgb_hitlist_count.restype = I64
    lib.cmgb_hitlist_get.argtypes = [P, I64, ctypes.POINTER(Hit)]
    lib.cmgb_hitlist_get.restype = I
    lib.cmgb_hitlist_clear.argtypes = [P]
    for name in ("cmgb_FastCYKScan", "cmgb_FastIInsideScan", "cmgb_FastCYKScan_dev", "cmgb_FastIInsideScan_dev",
                 "cmgb_FastFInsideScan", "cmgb_FastFInsideScan_dev"):
        f = getattr(lib, name)
        f.argtypes = _SCAN_ARGS
        f.restype = I
    for name in ("cmgb_RefTrCYKScan", "cmgb_RefITrInsideScan", "cmgb_RefTrCYKScan_dev", "cmgb_RefITrInsideScan_dev"):
        f = getattr(lib, name)
        f.argtypes = _TR_SCAN_ARGS
        f.restype = I
    lib.cmgb_ScanBatch.argtypes = [P, P, ctypes.c_char_p, I, I, I, P, I64, P, P, I, F, P, I, F, P, P, P, P, P]
    lib.cmgb_ScanBatch.restype = I
    lib.cmgb_ScanBatch_dev.argtypes = lib.cmgb_ScanBatch.argtypes
    lib.cmgb_ScanBatch_dev.restype = I
    lib.cmgb_ScanMulti.argtypes = [P, P, I, P, ctypes.c_char_p, I, I, P, I64, P, P, I, P, P, I, P, I, F, P, P, P, P]
    lib.cmgb_ScanMulti.restype = I
    lib.cmgb_ScanMulti_dev.argtypes = lib.cmgb_ScanMulti.argtypes
    lib.cmgb_ScanMulti_dev.restype = I
    lib.cmgb_Calibrate.argtypes = [P, P, ctypes.c_char_p, I, I64, I64, ctypes.c_uint64, I, P, P]
    lib.cmgb_Calibrate.restype = I
    lib.cmgb_filter_trainer_create.argtypes = [P, I, I, ctypes.c_uint64, ctypes.POINTER(P), ctypes.c_char_p]
    lib.cmgb_filter_trainer_create.restype = I
    lib.cmgb_filter_trainer_destroy.argtypes = [P]
    lib.cmgb_filter_trainer_destroy.restype = None
    lib.cmgb_filter_trainer_set.argtypes = [P, P, P, P, P, ctypes.c_char_p]
    lib.cmgb_filter_trainer_set.restype = I
    lib.cmgb_filter_trainer_step.argtypes = [P, P, P, F, F, F, P, P, ctypes.c_char_p]
    lib.cmgb_filter_trainer_step.restype = I
    lib.cmgb_filter_trainer_get.argtypes = [P, P, P, P, P, P, P, P, P, ctypes.c_char_p]
    lib.cmgb_filter_trainer_get.restype = I
    lib.cmgb_filter_create.argtypes = [P, I, P, P, P, P, ctypes.POINTER(P), ctypes.c_char_p]
    lib.cmgb_filter_create.restype = I
    lib.cmgb_filter_destroy.argtypes = [P]
    lib.cmgb_filter_windows.argtypes = [P, P, P, I64, I64, P, I64, ctypes.POINTER(I64), ctypes.POINTER(F), ctypes.c_char_p]
    lib.cmgb_filter_windows.restype = I
    lib.cmgb_filter_create_heads.argtypes = [P, I, I, P, P, P, P, ctypes.POINTER(P), ctypes.c_char_p]
    lib.cmgb_filter_create_heads.restype = I
    lib.cmgb_filter_trainer_create_heads.argtypes = [P, I, I, I, ctypes.c_uint64, ctypes.POINTER(P), ctypes.c_char_p]
    lib.cmgb_filter_trainer_create_heads.restype = I
    lib.cmgb_filter_trainer_step_heads.argtypes = [P, P, P, P, F, F, P, P, ctypes.c_char_p]
    lib.cmgb_filter_trainer_step_heads.restype = I
    lib.cmgb_measure_issue_peak.argtypes = [P, I, ctypes.POINTER(ctypes.c_double), ctypes.c_char_p]
    lib.cmgb_measure_issue_peak.restype = I
    lib.cmgb_autotune.argtypes = [P, P, I, I, I64, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.c_char_p]
    lib.cmgb_autotune.restype = I
    lib.cmgb_FastCYKScan_noalloc.argtypes = [P, P, ctypes.c_char_p, I, P, I64, I64, F, F, P, I, ctypes.POINTER(I),
                                             ctypes.POINTER(I64), ctypes.POINTER(I64), ctypes.POINTER(F)]
    lib.cmgb_FastCYKScan_noalloc.restype = I
    lib.cmgb_count_cells.argtypes = [P, I, I64]
    lib.cmgb_count_cells.restype = I64
    lib.cmgb_logsum_init()
    _libs[path] = lib
    return lib


def load(path: Optional[str] = None) -> ctypes.CDLL:
    """Loads the built GPU library; raises if it has not been built."""
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build it with __graft_entry__.build()")
    return bind(path)


class ExpInfo(ctypes.Structure):
    """cmgb_expinfo: the fields of a CM file ECM line."""
    _fields_ = [("lambda_", ctypes.c_double), ("mu_extrap", ctypes.c_double), ("mu_orig", ctypes.c_double),
                ("dbsize", ctypes.c_double), ("nrandhits", ctypes.c_int64), ("tailp", ctypes.c_double)]


def evalue(ecm, score: float, Z: float) -> float:
    """E-value of a bit score in a search of Z residues from an ECM line
    (lambda, mu_extrap, mu_orig, dbsize, nrandhits, tailp): Z / dbsize *
    nrandhits * exp(-lambda (S - mu_extrap))."""
    lam, mu_x, _mu, db, nrand, _tailp = ecm
    return Z / db * nrand * float(np.exp(-lam * (score - mu_x)))


def bits_at_evalue(ecm, E: float, Z: float) -> float:
    """The bit score whose E-value is E in a search of Z residues."""
    lam, mu_x, _mu, db, nrand, _tailp = ecm
    return mu_x - float(np.log(E / (Z / db * nrand))) / lam


@dataclass
class ScanResult:
    hits: List[tuple]          # (start, stop, root, mode, score)
    envi: int
    envj: int
    sc: float
    vsc: Optional[np.ndarray]
    kernel_ms: float
    mode: int = 3              # truncated scans: CMGB_TRMODE_* of the best parse


class Scanner:
    """One device context (the GB300 analogue of a worker's CM_SCAN_MX)."""

    def __init__(self, device: int = 0, lib: Optional[ctypes.CDLL] = None):
        self.lib = lib or load()
        self._ctx = P()
        err = ctypes.create_string_buffer(256)
        st = self.lib.cmgb_ctx_create(device, ctypes.byref(self._ctx), err)
        if st != 0:
            raise ScanError(st, err.value.decode())
        self._models = {}

    def close(self):
        for mh, _ in self._models.values():
            self.lib.cmgb_model_destroy(mh)
        self._models = {}
        if self._ctx:
            self.lib.cmgb_ctx_destroy(self._ctx)
            self._ctx = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_shape(self, tile_rows: int = 0, window_len: int = 0, ctas_per_sm: int = 0, threads: int = 0, arena: int = 0):
        st = self.lib.cmgb_ctx_set_shape(self._ctx, tile_rows, window_len, ctas_per_sm, threads, arena)
        if st != 0:
            raise ScanError(st, "invalid launch shape")

    def model(self, m: cmfile.CMModel, flags_extra: int = 0):
        key = (id(m), flags_extra)
        if key not in self._models:
            keep: list = []
            desc = cmfile.make_desc(m, flags_extra=flags_extra, keep=keep)
            h = P()
            err = ctypes.create_string_buffer(256)
            st = self.lib.cmgb_model_create(self._ctx, ctypes.byref(desc), ctypes.byref(h), err)
            if st != 0:
                raise ScanError(st, err.value.decode())
            self._models[key] = (h, (desc, keep, m))
        return self._models[key][0]

    def scan(self, m: cmfile.CMModel, dsq, i0: int, j0: int, algo: str = "cyk", qdbidx: int = 1,
             cutoff: float = 0.0, do_null3: bool = True, env_cutoff: float = 0.0, want_hits: bool = True,
             want_vsc: bool = False, notgreedy: bool = False, device_ptr: Optional[int] = None) -> ScanResult:
        """Runs cmgb_FastCYKScan (algo="cyk"), cmgb_FastIInsideScan (algo="inside") or
        cmgb_FastFInsideScan (algo="finside").
        dsq: numpy uint8 Easel digital sequence (dsq[0], dsq[L+1] sentinels);
        device_ptr: optional device address of the same array (the *_dev entry points)."""
        mh = self.model(m, CMGB_NOTGREEDY if notgreedy else 0)
        fn = {"cyk": "cmgb_FastCYKScan", "inside": "cmgb_FastIInsideScan", "finside": "cmgb_FastFInsideScan"}[algo]
        if device_ptr is not None:
            fn += "_dev"
            dptr = device_ptr
        else:
            dsq = np.ascontiguousarray(dsq, dtype=np.uint8)
            dptr = dsq.ctypes.data
        hl = self.lib.cmgb_hitlist_create() if want_hits else None
        envi, envj, sc = I64(), I64(), F()
        vsc = np.zeros(m.M, np.float32) if want_vsc else None
        err = ctypes.create_string_buffer(256)
        try:
            st = getattr(self.lib, fn)(self._ctx, mh, err, qdbidx, dptr, i0, j0, cutoff, hl,
                                       int(do_null3), env_cutoff, ctypes.byref(envi), ctypes.byref(envj),
                                       vsc.ctypes.data if vsc is not None else None, ctypes.byref(sc))
            if st != 0:
                raise ScanError(st, err.value.decode())
            hits = []
            if hl:
                h = Hit()
                for k in range(self.lib.cmgb_hitlist_count(hl)):
                    self.lib.cmgb_hitlist_get(hl, k, ctypes.byref(h))
                    hits.append((h.start, h.stop, h.root, h.mode, h.score))
        finally:
            if hl:
                self.lib.cmgb_hitlist_destroy(hl)
        return ScanResult(hits, envi.value, envj.value, sc.value, vsc,
                          float(self.lib.cmgb_ctx_last_kernel_ms(self._ctx)))

    def tr_scan(self, m: cmfile.CMModel, dsq, i0: int, j0: int, algo: str = "trcyk", qdbidx: int = 1,
                pass_idx: int = 4, cutoff: float = 0.0, do_null3: bool = True, env_cutoff: float = 0.0,
                want_hits: bool = True, want_vsc: bool = False, notgreedy: bool = False,
                device_ptr: Optional[int] = None) -> ScanResult:
        """Runs cmgb_RefTrCYKScan (algo="trcyk") or cmgb_RefITrInsideScan
        (algo="trinside") for pipeline pass pass_idx (2..5); the result's
        .mode is the mode of the best parse."""
        mh = self.model(m, CMGB_NOTGREEDY if notgreedy else 0)
        fn = TR_ALGOS[algo]
        if device_ptr is not None:
            fn += "_dev"
            dptr = device_ptr
        else:
            dsq = np.ascontiguousarray(dsq, dtype=np.uint8)
            dptr = dsq.ctypes.data
        hl = self.lib.cmgb_hitlist_create() if want_hits else None
        envi, envj, sc, mode = I64(), I64(), F(), I()
        vsc = np.zeros(m.M, np.float32) if want_vsc else None
        err = ctypes.create_string_buffer(256)
        try:
            st = getattr(self.lib, fn)(self._ctx, mh, err, qdbidx, pass_idx, dptr, i0, j0, cutoff, hl,
                                       int(do_null3), env_cutoff, ctypes.byref(envi), ctypes.byref(envj),
                                       vsc.ctypes.data if vsc is not None else None, ctypes.byref(mode),
                                       ctypes.byref(sc))
            if st != 0:
                raise ScanError(st, err.value.decode())
            hits = []
            if hl:
                h = Hit()
                for k in range(self.lib.cmgb_hitlist_count(hl)):
                    self.lib.cmgb_hitlist_get(hl, k, ctypes.byref(h))
                    hits.append((h.start, h.stop, h.root, h.mode, h.score))
        finally:
            if hl:
                self.lib.cmgb_hitlist_destroy(hl)
        return ScanResult(hits, envi.value, envj.value, sc.value, vsc,
                          float(self.lib.cmgb_ctx_last_kernel_ms(self._ctx)), mode.value)

    def scan_batch(self, m: cmfile.CMModel, seqs, algo: str = "cyk", qdbidx: int = 1, pass_idx: int = 4,
                   cutoff: float = 0.0, do_null3: bool = True, env_cutoff: float = 0.0, want_hits: bool = True,
                   notgreedy: bool = False, ranges=None, device_buf=None) -> List[ScanResult]:
        """Runs cmgb_ScanBatch over a list of digital sequences (each an Easel
        dsq with sentinels), scanning each over [1, L]; returns one
        ScanResult per sequence (vsc is None).
        ranges: instead of seqs, (buffer, offsets, lengths) -- sequences that
        are sub-ranges of one residue buffer (sequence q: residues
        buffer[offsets[q] + 1 .. offsets[q] + lengths[q]]);
        device_buf: (device address, length) of that buffer already in device
        memory (cmgb_ScanBatch_dev); buffer may then be None."""
        mh = self.model(m, CMGB_NOTGREEDY if notgreedy else 0)
        if ranges is not None:
            buf, offs, lens = ranges
            offs = np.ascontiguousarray(offs, np.int64)
            lens = np.ascontiguousarray(lens, np.int64)
            nseq = len(offs)
        else:
            parts = [np.ascontiguousarray(x, dtype=np.uint8) for x in seqs]
            lens = np.array([len(x) - 2 for x in parts], np.int64)
            offs = np.zeros(len(parts), np.int64)
            if len(parts) > 1:
                offs[1:] = np.cumsum([len(x) for x in parts[:-1]])
            buf = np.concatenate(parts + [np.full(1, cmfile.DSQ_SENTINEL, np.uint8)])
            nseq = len(parts)
        if nseq == 0:
            return []
        nh, ei, ej = np.zeros(nseq, np.int64), np.zeros(nseq, np.int64), np.zeros(nseq, np.int64)
        sc, mode = np.zeros(nseq, np.float32), np.zeros(nseq, np.int32)
        hl = self.lib.cmgb_hitlist_create() if want_hits else None
        err = ctypes.create_string_buffer(256)
        try:
            if device_buf is not None:
                fn, ptr, blen = self.lib.cmgb_ScanBatch_dev, device_buf[0], device_buf[1]
            else:
                fn, ptr, blen = self.lib.cmgb_ScanBatch, buf.ctypes.data, len(buf)
            st = fn(self._ctx, mh, err, BATCH_ALGOS[algo], qdbidx, pass_idx, ptr, blen, offs.ctypes.data, lens.ctypes.data,
                    nseq, cutoff, hl, int(do_null3), env_cutoff, nh.ctypes.data, ei.ctypes.data, ej.ctypes.data,
                    sc.ctypes.data, mode.ctypes.data)
            if st != 0:
                raise ScanError(st, err.value.decode())
            allhits = []
            if hl:
                h = Hit()
                for k in range(self.lib.cmgb_hitlist_count(hl)):
                    self.lib.cmgb_hitlist_get(hl, k, ctypes.byref(h))
                    allhits.append((h.start, h.stop, h.root, h.mode, h.score))
        finally:
            if hl:
                self.lib.cmgb_hitlist_destroy(hl)
        ms = float(self.lib.cmgb_ctx_last_kernel_ms(self._ctx))
        out, k = [], 0
        for q in range(nseq):
            out.append(ScanResult(allhits[k: k + int(nh[q])], int(ei[q]), int(ej[q]), float(sc[q]), None, ms, int(mode[q])))
            k += int(nh[q])
        return out

    def scan_multi(self, models, seqs, jobs=None, algo: str = "cyk", qdbidx: int = 1, cutoffs=None,
                   do_null3: bool = True, env_cutoff: float = 0.0, want_hits: bool = True,
                   ranges=None, device_buf=None) -> List[ScanResult]:
        """Runs cmgb_ScanMulti: every (model index, sequence index) pair of
        jobs (default: all models x all sequences) in one persistent launch per
        tile placement; returns one ScanResult per job, in job order.
        ranges / device_buf: sequences as sub-ranges of one residue buffer, as
        in scan_batch (cmgb_ScanMulti_dev when the buffer is on the device)."""
        if algo not in ("cyk", "inside", "finside"):
            raise ValueError("scan_multi runs the standard scanners only")
        mhs = [self.model(m, 0) for m in models]
        nm = len(models)
        if ranges is not None:
            buf, offs, lens = ranges
            offs = np.ascontiguousarray(offs, np.int64)
            lens = np.ascontiguousarray(lens, np.int64)
            nseq = len(offs)
        else:
            parts = [np.ascontiguousarray(x, dtype=np.uint8) for x in seqs]
            lens = np.array([len(x) - 2 for x in parts], np.int64)
            offs = np.zeros(len(parts), np.int64)
            if len(parts) > 1:
                offs[1:] = np.cumsum([len(x) for x in parts[:-1]])
            buf = np.concatenate(parts + [np.full(1, cmfile.DSQ_SENTINEL, np.uint8)])
            nseq = len(parts)
        if jobs is None:
            jobs = [(a, b) for a in range(nm) for b in range(nseq)]
        jm = np.array([a for a, _ in jobs], np.int32)
        js = np.array([b for _, b in jobs], np.int32)
        nj = len(jobs)
        cut = np.asarray(cutoffs if cutoffs is not None else [0.0] * nm, np.float32)
        harr = (ctypes.c_void_p * nm)(*[h.value for h in mhs])
        nh, ei, ej = np.zeros(nj, np.int64), np.zeros(nj, np.int64), np.zeros(nj, np.int64)
        sc = np.zeros(nj, np.float32)
        hl = self.lib.cmgb_hitlist_create() if want_hits else None
        err = ctypes.create_string_buffer(256)
        try:
            if nj == 0:
                return []
            if device_buf is not None:
                fn, ptr, blen = self.lib.cmgb_ScanMulti_dev, device_buf[0], device_buf[1]
            else:
                fn, ptr, blen = self.lib.cmgb_ScanMulti, buf.ctypes.data, len(buf)
            st = fn(self._ctx, harr, nm, cut.ctypes.data, err, BATCH_ALGOS[algo], qdbidx, ptr, blen, offs.ctypes.data,
                    lens.ctypes.data, nseq, jm.ctypes.data, js.ctypes.data, nj, hl, int(do_null3), env_cutoff,
                    nh.ctypes.data, ei.ctypes.data, ej.ctypes.data, sc.ctypes.data)
            if st != 0:
                raise ScanError(st, err.value.decode())
            allhits = []
            if hl:
                h = Hit()
                for k in range(self.lib.cmgb_hitlist_count(hl)):
                    self.lib.cmgb_hitlist_get(hl, k, ctypes.byref(h))
                    allhits.append((h.start, h.stop, h.root, h.mode, h.score))
        finally:
            if hl:
                self.lib.cmgb_hitlist_destroy(hl)
        ms = float(self.lib.cmgb_ctx_last_kernel_ms(self._ctx))
        out, k = [], 0
        for q in range(nj):
            out.append(ScanResult(allhits[k: k + int(nh[q])], int(ei[q]), int(ej[q]), float(sc[q]), None, ms, 0))
            k += int(nh[q])
        return out

    def calibrate(self, m: cmfile.CMModel, algo: str = "cyk", total_len: int = 1_600_000, seq_len: int = 100_000,
                  seed: int = 181, tail_per_mb: int = 750):
        """Runs cmgb_Calibrate; returns (ExpInfo as the CM file's ECM fields, kernel ms)."""
        mh = self.model(m, 0)
        e = ExpInfo()
        ms = ctypes.c_float()
        err = ctypes.create_string_buffer(256)
        st = self.lib.cmgb_Calibrate(self._ctx, mh, err, BATCH_ALGOS[{"cyk": "cyk", "inside": "inside"}[algo]],
                                     total_len, seq_len, seed, tail_per_mb, ctypes.byref(e), ctypes.byref(ms))
        if st != 0:
            raise ScanError(st, err.value.decode())
        return (e.lambda_, e.mu_extrap, e.mu_orig, e.dbsize, float(e.nrandhits), e.tailp), ms.value

    def autotune(self, m: cmfile.CMModel, qdbidx: int, algo: str = "cyk", sample_len: int = 0):
        """Runs cmgb_autotune for (model, band set, algorithm); returns (tile_rows, arena)."""
        mh = self.model(m, 0)
        t, a = I(), I()
        err = ctypes.create_string_buffer(256)
        st = self.lib.cmgb_autotune(self._ctx, mh, qdbidx, {"cyk": 0, "inside": 1, "finside": 2}[algo], sample_len,
                                    ctypes.byref(t), ctypes.byref(a), err)
        if st != 0:
            raise ScanError(st, err.value.decode())
        return t.value, a.value

    def last_transfer_bytes(self):
        """(host->device, device->host) bytes moved by the last scan."""
        a, b = I64(), I64()
        self.lib.cmgb_ctx_last_transfer_bytes(self._ctx, ctypes.byref(a), ctypes.byref(b))
        return a.value, b.value

    def issue_peak(self, kind: str = "f32") -> float:
        """Measured arithmetic issue rate of this device (operations per second,
        add and max counted separately) for the fp32 ("f32") or int32 ("i32")
        add + max pair: the scan kernels' roofline denominator."""
        v = ctypes.c_double()
        err = ctypes.create_string_buffer(256)
        st = self.lib.cmgb_measure_issue_peak(self._ctx, {"f32": 0, "i32": 1}[kind], ctypes.byref(v), err)
        if st != 0:
            raise ScanError(st, err.value.decode())
        return v.value

    def last_launches(self) -> int:
        return int(self.lib.cmgb_ctx_last_launches(self._ctx))
