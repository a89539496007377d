"""CPU oracle for the sDTW read-classification path.

TEST INFRASTRUCTURE ONLY: the oracle the CUDA library is compared against.
Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module.  The product package (dtwax_gb300) never imports it.

Two independent restatements of the reference algorithm live here:

* ``liboracle.so`` (sdtw_oracle.c): FP64 OpenMP C, used for every parity check
  and for the timed CPU baseline;
* small numpy versions (``np_sdtw``, ``np_zscore``, ``np_build_levels``,
  ``np_best_threshold``) used to cross-check the C code on small cases.

Reference files followed (paths inside harisankarsadasivan/DTWax):
scripts/sdtw.py:86-116 and :205-225, src/include/DTW.cu:37-39,
src/include/load_reference.hpp:33-128, src/include/normalizer.cu:397-399,
src/ReadUntil/calc_classification_threshold.py:49-57, and for the reference
kernel's own evaluation order src/include/DTW.cu:151-572.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")
SRC_PATH = os.path.join(HERE, "sdtw_oracle.c")

_lib = None

_d = ctypes.POINTER(ctypes.c_double)
_i64 = ctypes.POINTER(ctypes.c_int64)


def build(force: bool = False) -> str:
    """Compile liboracle.so with gcc (OpenMP, no FP contraction)."""
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC_PATH):
        return LIB_PATH
    cmd = ["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-shared", "-fPIC",
           SRC_PATH, "-o", LIB_PATH + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(LIB_PATH + ".tmp", LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.oracle_zscore.argtypes = [_d, ctypes.c_int64, ctypes.c_double, _d]
        L.oracle_zscore.restype = ctypes.c_int64
        L.oracle_build_levels.argtypes = [ctypes.c_char_p, ctypes.c_int64, _d, ctypes.c_int64, _d, _d]
        L.oracle_build_levels.restype = ctypes.c_int64
        L.oracle_sdtw.argtypes = [_d, ctypes.c_int64, _d, ctypes.c_int64, _d, _d, _i64,
                                  _i64, ctypes.c_int, _d]
        L.oracle_sdtw.restype = ctypes.c_double
        L.oracle_sdtw_batch.argtypes = [_d, _d, ctypes.c_int64, _d, _i64, ctypes.c_int,
                                        _d, _i64, _d, _i64, ctypes.c_int]
        L.oracle_sdtw_batch.restype = None
        L.oracle_sdtw_ref_del.argtypes = [_d, ctypes.c_int64, _d, ctypes.c_int64, _d, _d, _i64]
        L.oracle_sdtw_ref_del.restype = ctypes.c_double
        L.oracle_sdtw_batch_rec.argtypes = [_d, _d, ctypes.c_int64, _d, _i64, ctypes.c_int,
                                            _d, _i64, _d, _i64, ctypes.c_int, ctypes.c_int]
        L.oracle_sdtw_batch_rec.restype = None
        L.oracle_sdtw_refkernel.argtypes = [_d, ctypes.c_int64, _d, ctypes.c_int64, ctypes.c_int]
        L.oracle_sdtw_refkernel.restype = ctypes.c_double
        L.oracle_sdtw_refkernel_batch.argtypes = [_d, ctypes.c_int64, _d, ctypes.c_int64, ctypes.c_int,
                                                  ctypes.c_int, _d, ctypes.c_int]
        L.oracle_sdtw_refkernel_batch.restype = None
        L.oracle_max_threads.argtypes = []
        L.oracle_max_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(_d)


def _ip(a):
    return a.ctypes.data_as(_i64)


# ---------------------------------------------------------------- C oracle

def zscore(x, eps: float = 0.0) -> np.ndarray:
    x = np.ascontiguousarray(x, dtype=np.float64)
    y = np.empty_like(x)
    lib().oracle_zscore(_dp(x), x.size, float(eps), _dp(y))
    return y


def build_levels(seq: bytes, table, cap: int = 0):
    """(fwd, rev) z-scored 6-mer levels of both strands, FP64."""
    table = np.ascontiguousarray(table, dtype=np.float64)
    assert table.size == 4096
    L = len(seq)
    m = max(L - 5, 0)
    if cap and cap < m:
        m = cap
    fwd = np.empty(max(m, 1), np.float64)
    rev = np.empty(max(m, 1), np.float64)
    got = lib().oracle_build_levels(seq, L, _dp(table), int(cap), _dp(fwd), _dp(rev))
    assert got == m, (got, m)
    return fwd[:m], rev[:m]


def sdtw(ref, q, init_row=None, trace_cols=None, want_row: bool = False):
    """FP64 sDTW of one query against one sequence.

    Returns (score, argmin) or (score, argmin, trace) when trace_cols is given;
    with want_row the final DP row is appended."""
    ref = np.ascontiguousarray(ref, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    am = np.zeros(1, np.int64)
    init = None
    if init_row is not None:
        init = np.ascontiguousarray(init_row, dtype=np.float64)
        assert init.size == ref.size
    row = np.empty(ref.size, np.float64) if want_row else None
    tc = None
    tr = None
    nt = 0
    if trace_cols is not None:
        tc = np.ascontiguousarray(trace_cols, dtype=np.int64)
        nt = tc.size
        tr = np.empty((q.size, nt), np.float64)
    s = lib().oracle_sdtw(_dp(ref), ref.size, _dp(q), q.size,
                          _dp(init) if init is not None else None,
                          _dp(row) if row is not None else None, _ip(am),
                          _ip(tc) if tc is not None else None, nt,
                          _dp(tr) if tr is not None else None)
    out = [float(s), int(am[0])]
    if trace_cols is not None:
        out.append(tr)
    if want_row:
        out.append(row)
    return tuple(out)


def sdtw_ref_del(ref, q, init_row=None, want_row: bool = False):
    """FP64 sDTW with the REF_DEL recurrence (a left predecessor in the same
    row, DTW.cu:23-29): (score, argmin[, final row])."""
    ref = np.ascontiguousarray(ref, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    am = np.zeros(1, np.int64)
    init = None if init_row is None else np.ascontiguousarray(init_row, dtype=np.float64)
    row = np.empty(ref.size, np.float64) if want_row else None
    s = lib().oracle_sdtw_ref_del(_dp(ref), ref.size, _dp(q), q.size, _dp(init) if init is not None else None,
                                  _dp(row) if row is not None else None, _ip(am))
    return (float(s), int(am[0]), row) if want_row else (float(s), int(am[0]))


def sdtw_batch(fwd, rev, queries, offsets, n_threads: int = 0, ref_del: bool = False):
    """Per read: (score_fwd, end_fwd, score_rev, end_rev) arrays, FP64, OpenMP;
    ref_del selects the REF_DEL recurrence."""
    fwd = np.ascontiguousarray(fwd, dtype=np.float64)
    rev = np.ascontiguousarray(rev, dtype=np.float64)
    assert fwd.size == rev.size
    queries = np.ascontiguousarray(queries, dtype=np.float64)
    offsets = np.ascontiguousarray(offsets, dtype=np.int64)
    n = offsets.size - 1
    sf = np.empty(n, np.float64)
    sr = np.empty(n, np.float64)
    ef = np.empty(n, np.int64)
    er = np.empty(n, np.int64)
    if n > 0:
        lib().oracle_sdtw_batch_rec(_dp(fwd), _dp(rev), fwd.size, _dp(queries), _ip(offsets), n,
                                    _dp(sf), _ip(ef), _dp(sr), _ip(er), int(n_threads), int(bool(ref_del)))
    return sf, ef, sr, er


# Departures of the reference GPU kernel from the recurrence (src/include/DTW.cu),
# switches of oracle_sdtw_refkernel; see sdtw_oracle.c for each.
REFK_TILE = 832
REFK_CHUNK = 1024
REFK_CHUNK_SEAM_DIAG = 1
REFK_CHUNK_LANE1_DIAG = 2
REFK_SEAM_SHIFT = 4
REFK_ALL = 7
REFK_REF_DEL = 8  # the REF_DEL recurrence (not a departure)


def sdtw_refkernel(ref, q, quirks: int = REFK_ALL) -> float:
    """min over the last row in the reference kernel's tile/chunk order with
    the chosen departures; ref holds whole 832-column tiles, q 1,024-row chunks."""
    ref = np.ascontiguousarray(ref, dtype=np.float64)
    q = np.ascontiguousarray(q, dtype=np.float64)
    return float(lib().oracle_sdtw_refkernel(_dp(ref), ref.size, _dp(q), q.size, int(quirks)))


def sdtw_refkernel_batch(ref, queries, quirks: int = REFK_ALL, n_threads: int = 0):
    """sdtw_refkernel for each row of the 2-D array queries (OpenMP)."""
    ref = np.ascontiguousarray(ref, dtype=np.float64)
    queries = np.ascontiguousarray(queries, dtype=np.float64)
    n, qlen = queries.shape
    out = np.empty(n, np.float64)
    if n > 0:
        lib().oracle_sdtw_refkernel_batch(_dp(ref), ref.size, _dp(queries), qlen, n, int(quirks),
                                          _dp(out), int(n_threads))
    return out


def max_threads() -> int:
    return int(lib().oracle_max_threads())


def combine(sf, ef, sr, er):
    """Per-read best hit with the tie rule: lowest score, then smallest end
    column, then forward before reverse.  Returns (score, end, strand)."""
    sf = np.asarray(sf); sr = np.asarray(sr)
    ef = np.asarray(ef); er = np.asarray(er)
    pick_rev = (sr < sf) | ((sr == sf) & (er < ef))
    score = np.where(pick_rev, sr, sf)
    end = np.where(pick_rev, er, ef)
    return score, end, pick_rev.astype(np.int8)


# ---------------------------------------------------------------- numpy versions

def np_zscore(x, eps: float = 0.0):
    """sdtw.py:97-99 (eps 0) / normalizer.cu:397-399 (eps 1e-4)."""
    x = np.asarray(x, dtype=np.float64)
    mean = np.mean(x)
    return (x - mean) / np.sqrt(np.mean((x - mean) ** 2) + eps)


def np_kmer_codes(seq: bytes) -> np.ndarray:
    lut = np.full(256, -1, np.int64)
    for ch, v in ((b"A", 0), (b"C", 1), (b"G", 2), (b"T", 3), (b"a", 0), (b"c", 1), (b"g", 2), (b"t", 3)):
        lut[ch[0]] = v
    b = lut[np.frombuffer(seq, np.uint8)]
    m = len(seq) - 5
    if m <= 0:
        return np.zeros(0, np.int64)
    code = np.zeros(m, np.int64)
    bad = np.zeros(m, bool)
    for k in range(6):
        part = b[k:k + m]
        bad |= part < 0
        code = code * 4 + np.maximum(part, 0)
    code[bad] = -1
    return code


def np_revcomp(seq: bytes) -> bytes:
    tr = bytes.maketrans(b"ACGTacgt", b"TGCAtgca")
    return seq.translate(tr)[::-1]


def np_build_levels(seq: bytes, table, cap: int = 0):
    table = np.asarray(table, dtype=np.float64)
    out = []
    for s in (seq, np_revcomp(seq)):
        c = np_kmer_codes(s)
        if cap and cap < c.size:
            c = c[:cap]
        lv = np.where(c >= 0, table[np.maximum(c, 0)], np.nan)
        ok = ~np.isnan(lv)
        z = np.zeros_like(lv)
        if ok.any():
            v = lv[ok]
            mean = v.mean()
            z[ok] = (v - mean) / np.sqrt(np.mean((v - mean) ** 2))
        out.append(z)
    return out[0], out[1]


def np_sdtw(ref, q, init_row=None, ref_del: bool = False):
    """Row-vectorised FP64 sDTW for small cases (sdtw.py:205-225); ref_del
    adds the left predecessor (DTW.cu:23-29) with a plain loop along the row."""
    ref = np.asarray(ref, dtype=np.float64)
    q = np.asarray(q, dtype=np.float64)
    prev = np.zeros(ref.size) if init_row is None else np.array(init_row, dtype=np.float64)
    for qi in q:
        cost = (ref - qi) ** 2
        cur = np.empty_like(prev)
        cur[0] = cost[0] + prev[0]
        cur[1:] = cost[1:] + np.minimum(prev[1:], prev[:-1])
        if ref_del:
            for j in range(1, ref.size):
                cur[j] = min(cur[j], cost[j] + cur[j - 1])
        prev = cur
    j = int(np.argmin(prev))
    return float(prev[j]), j, prev


def np_best_threshold(target_scores, other_scores, num: int = 100000):
    """calc_classification_threshold.py:49-57: sweep linspace(0, max, num) and
    keep the first threshold of maximal accuracy, where a target read is
    correct when score < t and a non-target read when score >= t."""
    t_s = np.asarray(target_scores, dtype=np.float64)
    o_s = np.asarray(other_scores, dtype=np.float64)
    th = np.linspace(0, max(t_s.max(), o_s.max()), num=num)
    ts = np.sort(t_s)
    os_ = np.sort(o_s)
    correct_t = np.searchsorted(ts, th, side="left")          # count(score < t)
    correct_o = os_.size - np.searchsorted(os_, th, side="left")  # count(score >= t)
    acc = (correct_t + correct_o) * 100.0 / (t_s.size + o_s.size)
    k = int(np.argmax(acc))
    return float(th[k]), float(acc[k])
