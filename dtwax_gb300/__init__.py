"""dtwax_gb300 -- GB300-native subsequence-DTW nanopore read classifier.

Python face of libdtwx.so (include/dtwx.h).  Everything that computes runs in
the CUDA library; this module only moves arrays across the C ABI.  There is no
CPU fallback: if the library has not been built, importing succeeds but
creating a Classifier raises.

Reference interface mirrored (harisankarsadasivan/DTWax):
  load_reference (src/include/load_reference.hpp:14-212)  -> Classifier(...)
  normalizer::normalize (src/include/normalizer.cu:370-413) +
  FullDTW::distances (src/include/DTW.hpp:287-295)        -> Classifier.classify / .distances
  main log (src/main.cu:279-299)                          -> format_log
"""
from __future__ import annotations

import ctypes
import os
from typing import Iterable, Sequence

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libdtwx.so")
CLI_PATH = os.path.join(PKG, "bin", "dtwx_main")

DTWX_OK = 0
STATUS = {0: "OK", -1: "E_ARG", -2: "E_IO", -3: "E_FORMAT", -4: "E_CUDA", -5: "E_NOMEM",
          -6: "E_TIMEOUT", -7: "E_CAPACITY", -8: "E_STATE"}
FP16, FP32, MIXED = 0, 1, 2  # MIXED: FP16 differences, FP32 path cost
NO_REF_DEL, REF_DEL = 0, 1     # recurrence: without / with the left predecessor
STATE_FP32, STATE_FP16 = 0, 1  # serving row state
STRANDS_PAIRED, STRANDS_CONCAT = 0, 1
CALL_DEVICE_ERROR = -2  # dtwx_result.call of reads whose call hit a device-side error
ABI_VERSION = 2


class DtwxError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class Config(ctypes.Structure):
    _fields_ = [
        ("abi_version", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("strand_mode", ctypes.c_int32), ("device", ctypes.c_int32),
        ("max_ref_len", ctypes.c_int64), ("adapter_skip", ctypes.c_int32),
        ("query_len", ctypes.c_int32), ("require_full", ctypes.c_int32),
        ("norm_eps", ctypes.c_float), ("threshold", ctypes.c_float),
        ("max_batch_reads", ctypes.c_int32), ("cells_per_thread", ctypes.c_int32),
        ("chunk_strips", ctypes.c_int32), ("warps_per_cta", ctypes.c_int32),
        ("use_graphs", ctypes.c_int32), ("serve_batches", ctypes.c_int32), ("recurrence", ctypes.c_int32),
        ("state_precision", ctypes.c_int32), ("reserved", ctypes.c_int32 * 4),
    ]


class Result(ctypes.Structure):
    _fields_ = [("score", ctypes.c_float), ("score_fwd", ctypes.c_float), ("score_rev", ctypes.c_float),
                ("strand", ctypes.c_int32), ("end_pos", ctypes.c_int64), ("call", ctypes.c_int32),
                ("n_samples", ctypes.c_int32)]


class Decision(ctypes.Structure):
    _fields_ = [("channel", ctypes.c_int32), ("decided", ctypes.c_int32), ("read_number", ctypes.c_uint64),
                ("score", ctypes.c_float), ("strand", ctypes.c_int32), ("call", ctypes.c_int32),
                ("end_pos", ctypes.c_int64), ("chunks", ctypes.c_int32), ("samples", ctypes.c_int32),
                ("latency_ms", ctypes.c_double), ("queue_ms", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [("chunks_submitted", ctypes.c_int64), ("chunks_processed", ctypes.c_int64),
                ("reads_decided", ctypes.c_int64), ("reads_deferred", ctypes.c_int64),
                ("queue_depth", ctypes.c_int32), ("in_flight", ctypes.c_int32),
                ("max_in_flight", ctypes.c_int32), ("batches", ctypes.c_int32),
                ("p50_latency_ms", ctypes.c_double), ("p99_latency_ms", ctypes.c_double),
                ("mean_batch_reads", ctypes.c_double), ("state_bytes", ctypes.c_double),
                ("mean_batch_ms", ctypes.c_double), ("max_batch_ms", ctypes.c_double),
                ("p50_queue_ms", ctypes.c_double), ("p99_queue_ms", ctypes.c_double)]


# numpy view of dtwx_result (32 bytes)
RESULT_DTYPE = np.dtype([("score", "<f4"), ("score_fwd", "<f4"), ("score_rev", "<f4"), ("strand", "<i4"),
                         ("end_pos", "<i8"), ("call", "<i4"), ("n_samples", "<i4")])
assert RESULT_DTYPE.itemsize == ctypes.sizeof(Result) == 32

_lib = None

_P = ctypes.c_void_p
_I64P = ctypes.POINTER(ctypes.c_int64)

_SIGNATURES = {
    "dtwx_config_default": (ctypes.c_int, [ctypes.POINTER(Config)]),
    "dtwx_create": (ctypes.c_int, [ctypes.POINTER(Config), ctypes.c_char_p, _P, ctypes.c_char_p, ctypes.POINTER(_P)]),
    "dtwx_create_from_sequence": (ctypes.c_int, [ctypes.POINTER(Config), _P, ctypes.c_char_p, ctypes.c_int64,
                                                 ctypes.POINTER(_P)]),
    "dtwx_load_fasta": (ctypes.c_int, [ctypes.c_char_p, _P, ctypes.c_int64, _I64P]),
    "dtwx_load_kmer_model": (ctypes.c_int, [ctypes.c_char_p, _P]),
    "dtwx_destroy": (ctypes.c_int, [_P]),
    "dtwx_last_error": (ctypes.c_char_p, [_P]),
    "dtwx_ref_len": (ctypes.c_int64, [_P]),
    "dtwx_get_reference": (ctypes.c_int, [_P, _P, _P]),
    "dtwx_classify_batch": (ctypes.c_int, [_P, _P, _I64P, ctypes.c_int32, _P]),
    "dtwx_classify_batch_i16": (ctypes.c_int, [_P, _P, _I64P, ctypes.c_int32, _P, _P, _P, _P]),
    "dtwx_distances": (ctypes.c_int, [_P, _P, _I64P, ctypes.c_int32, _P, _P]),
    "dtwx_classify_device": (ctypes.c_int, [_P, _P, _I64P, ctypes.c_int32, _P, _P]),
    "dtwx_sync": (ctypes.c_int, [_P]),
    "dtwx_normalize": (ctypes.c_int, [_P, _P, _I64P, ctypes.c_int32, _P, _I64P, _P]),
    "dtwx_debug_stall_next": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_uint32]),
    "dtwx_classify_plain_fp32": (ctypes.c_int, [_P, _P, _I64P, ctypes.c_int32, _P]),
    "dtwx_distances_static": (ctypes.c_int, [_P, ctypes.c_int64, _P, _I64P, ctypes.c_int32, ctypes.c_float, _P, _P]),
    "dtwx_last_launch_count": (ctypes.c_int32, [_P]),
    "dtwx_last_sweep_ms": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float)]),
    "dtwx_autotune": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_float)]),
    "dtwx_get_tuning": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_int32), ctypes.c_int32]),
    "dtwx_peak_probe": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                                       ctypes.POINTER(ctypes.c_double)]),
    "dtwx_serve_start": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_double, ctypes.c_int32, ctypes.c_float,
                                        ctypes.c_float]),
    "dtwx_submit_chunk": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_uint64, _P, ctypes.c_int32, ctypes.c_int32,
                                         ctypes.c_double]),
    "dtwx_submit_chunk_i16": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_uint64, _P, ctypes.c_int32,
                                             ctypes.c_int32, ctypes.c_double, ctypes.c_float, ctypes.c_float,
                                             ctypes.c_float]),
    "dtwx_serve_step": (ctypes.c_int, [_P]),
    "dtwx_poll_decisions": (ctypes.c_int, [_P, ctypes.POINTER(Decision), ctypes.c_int32]),
    "dtwx_serve_drain": (ctypes.c_int, [_P]),
    "dtwx_stats_get": (ctypes.c_int, [_P, ctypes.POINTER(Stats)]),
    "dtwx_now_ms": (ctypes.c_double, []),
}


def load_library(path: str = LIB_PATH):
    """Load libdtwx.so (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"{path} is missing: build it with `python -m dtwax_gb300.build` "
                               "(the classifier has no CPU implementation)")
        L = ctypes.CDLL(path)
        for name, (res, args) in _SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc: int, handle=None):
    if rc < 0:
        msg = load_library().dtwx_last_error(handle).decode(errors="replace")
        raise DtwxError(rc, msg)
    return rc


def default_config(**overrides) -> Config:
    cfg = Config()
    load_library().dtwx_config_default(ctypes.byref(cfg))
    for k, v in overrides.items():
        if not hasattr(cfg, k):
            raise TypeError(f"unknown config field {k}")
        setattr(cfg, k, v)
    return cfg


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data)


def pack_reads(reads: Iterable[np.ndarray], dtype=np.float32):
    """List of 1-D sample arrays -> (concatenated samples, offsets[n+1])."""
    reads = [np.asarray(r) for r in reads]
    offsets = np.zeros(len(reads) + 1, np.int64)
    if reads:
        offsets[1:] = np.cumsum([r.size for r in reads])
    raw = np.concatenate([r.astype(dtype, copy=False) for r in reads]) if reads else np.zeros(0, dtype)
    return np.ascontiguousarray(raw, dtype=dtype), offsets


class Classifier:
    """sDTW classifier for one target genome on one GPU.

    Exactly one reference source: ``fasta`` (a FASTA path, parsed with the
    reference's single-record rules) or ``sequence`` (bases as str/bytes); and
    one level source: ``kmer_model`` (text "KMER mean stdev") or
    ``level_table`` (4096 means by 2-bit code).  Remaining keyword arguments set
    fields of :class:`Config`.
    """

    def __init__(self, fasta: str | None = None, kmer_model: str | None = None,
                 level_table: Sequence[float] | None = None, sequence: str | bytes | None = None, **cfg):
        L = load_library()
        self._lib = L
        self.cfg = default_config(**cfg)
        h = ctypes.c_void_p()
        self._table = None
        if level_table is not None:
            self._table = np.ascontiguousarray(level_table, dtype=np.float32)
            if self._table.size != 4096:
                raise ValueError("level_table needs 4096 entries")
        if sequence is not None:
            if self._table is None:
                raise ValueError("sequence= needs level_table=")
            seq = sequence.encode() if isinstance(sequence, str) else bytes(sequence)
            rc = L.dtwx_create_from_sequence(ctypes.byref(self.cfg), _ptr(self._table), seq, len(seq), ctypes.byref(h))
        else:
            if fasta is None:
                raise ValueError("give fasta= or sequence=")
            rc = L.dtwx_create(ctypes.byref(self.cfg), kmer_model.encode() if kmer_model else None,
                               _ptr(self._table) if self._table is not None else None, fasta.encode(),
                               ctypes.byref(h))
        _check(rc, None)
        self._h = h

    # -- lifetime
    def close(self):
        if getattr(self, "_h", None):
            self._lib.dtwx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- reference
    @property
    def ref_len(self) -> int:
        return int(self._lib.dtwx_ref_len(self._h))

    def reference(self):
        """z-scored squiggle of both strands, FP32 (fwd, rev)."""
        m = self.ref_len
        fwd = np.empty(m, np.float32)
        rev = np.empty(m, np.float32)
        _check(self._lib.dtwx_get_reference(self._h, _ptr(fwd), _ptr(rev)), self._h)
        return fwd, rev

    # -- offline classification
    def classify(self, reads=None, raw: np.ndarray | None = None, offsets: np.ndarray | None = None) -> np.ndarray:
        """Classify reads (list of arrays, or raw + offsets).  Returns a
        structured array of RESULT_DTYPE."""
        if reads is not None:
            raw, offsets = pack_reads(reads, np.float32)
        raw = np.ascontiguousarray(raw, dtype=np.float32)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        n = offsets.size - 1
        out = np.zeros(max(n, 0), RESULT_DTYPE)
        _check(self._lib.dtwx_classify_batch(self._h, _ptr(raw), offsets.ctypes.data_as(_I64P), n, _ptr(out)),
               self._h)
        return out

    def classify_i16(self, reads=None, raw=None, offsets=None, offset=None, range_=None, digitisation=None):
        if reads is not None:
            raw, offsets = pack_reads(reads, np.int16)
        raw = np.ascontiguousarray(raw, dtype=np.int16)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        n = offsets.size - 1
        f = [None if a is None else np.ascontiguousarray(a, dtype=np.float32) for a in (offset, range_, digitisation)]
        out = np.zeros(max(n, 0), RESULT_DTYPE)
        _check(self._lib.dtwx_classify_batch_i16(self._h, _ptr(raw), offsets.ctypes.data_as(_I64P), n,
                                                 *[(_ptr(a) if a is not None else None) for a in f], _ptr(out)),
               self._h)
        return out

    def classify_plain_fp32(self, reads=None, raw=None, offsets=None) -> np.ndarray:
        """One sDTW launch per read in FP32 (the plain comparator)."""
        if reads is not None:
            raw, offsets = pack_reads(reads, np.float32)
        raw = np.ascontiguousarray(raw, dtype=np.float32)
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        n = offsets.size - 1
        out = np.zeros(max(n, 0), RESULT_DTYPE)
        _check(self._lib.dtwx_classify_plain_fp32(self._h, _ptr(raw), offsets.ctypes.data_as(_I64P), n, _ptr(out)),
               self._h)
        return out

    def distances(self, d_query: int, offsets: np.ndarray, d_out: int, stream: int = 0):
        """Device-pointer entry (FullDTW::distances): d_query/d_out are device
        addresses, offsets a host int64 array; asynchronous on `stream`
        (a cudaStream_t value; 0 = the legacy default stream)."""
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        _check(self._lib.dtwx_distances(self._h, ctypes.c_void_p(d_query), offsets.ctypes.data_as(_I64P),
                                        offsets.size - 1, ctypes.c_void_p(d_out), ctypes.c_void_p(stream)), self._h)

    def classify_device(self, d_raw: int, offsets: np.ndarray, d_out: int, stream: int = 0):
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        _check(self._lib.dtwx_classify_device(self._h, ctypes.c_void_p(d_raw), offsets.ctypes.data_as(_I64P),
                                              offsets.size - 1, ctypes.c_void_p(d_out), ctypes.c_void_p(stream)),
               self._h)

    def normalize(self, d_raw: int, offsets: np.ndarray, d_query: int, stream: int = 0) -> np.ndarray:
        """Window + z-score of device-resident raw samples into d_query
        (normalizer::normalize); returns the output offsets (host)."""
        offsets = np.ascontiguousarray(offsets, dtype=np.int64)
        out = np.zeros(offsets.size, np.int64)
        _check(self._lib.dtwx_normalize(self._h, ctypes.c_void_p(d_raw), offsets.ctypes.data_as(_I64P),
                                        offsets.size - 1, ctypes.c_void_p(d_query), out.ctypes.data_as(_I64P),
                                        ctypes.c_void_p(stream)), self._h)
        return out

    def sync(self):
        """Wait for the last device-pointer call (distances / classify_device)
        and raise DtwxError if its kernels reported a device-side error."""
        _check(self._lib.dtwx_sync(self._h), self._h)

    def debug_stall_next(self, item: int, spin_limit: int = 0):
        """Test hook: the next sweep withholds the first reference-strip copy of
        work item `item`, so that item's bounded wait runs out (after
        spin_limit polls, 0 = the library's limit)."""
        _check(self._lib.dtwx_debug_stall_next(self._h, int(item), int(spin_limit)), self._h)

    @property
    def last_launch_count(self) -> int:
        return int(self._lib.dtwx_last_launch_count(self._h))

    def last_sweep_ms(self) -> float:
        """Device time of the last sDTW sweep kernel (CUDA events on its stream)."""
        v = ctypes.c_float()
        _check(self._lib.dtwx_last_sweep_ms(self._h, ctypes.byref(v)), self._h)
        return v.value

    def autotune(self, n_reads: int, read_len: int) -> float:
        """Time the candidate launch shapes on a synthetic batch of this size;
        returns the best sweep time in ms (the shape is kept for such batches)."""
        v = ctypes.c_float()
        _check(self._lib.dtwx_autotune(self._h, n_reads, read_len, ctypes.byref(v)), self._h)
        return v.value

    def tuning(self):
        """Launch shape of the most recent batched sweep."""
        v = (ctypes.c_int32 * 8)()
        _check(self._lib.dtwx_get_tuning(self._h, v, 8), self._h)
        keys = ("cells_per_thread", "chunk_strips", "warps_per_cta", "ctas", "work_items", "ctas_per_sm",
                "graph_replays", "narrow_halo")
        return dict(zip(keys, list(v)))

    # -- Read Until serving
    def serve_start(self, max_in_flight: int = 0, state_budget_bytes: float = 0.0, chunks_per_decision: int = 3,
                    accept_per_sample: float = 0.0, reject_per_sample: float = 0.0):
        _check(self._lib.dtwx_serve_start(self._h, max_in_flight, float(state_budget_bytes), chunks_per_decision,
                                          float(accept_per_sample), float(reject_per_sample)), self._h)

    def submit_chunk(self, channel: int, read_number: int, samples: np.ndarray, is_last: bool = False,
                     arrival_ms: float = -1.0):
        s = np.ascontiguousarray(samples, dtype=np.float32)
        _check(self._lib.dtwx_submit_chunk(self._h, channel, read_number, _ptr(s), s.size, int(is_last),
                                           float(arrival_ms)), self._h)

    def submit_chunk_i16(self, channel: int, read_number: int, samples: np.ndarray, offset: float,
                         range_: float, digitisation: float, is_last: bool = False, arrival_ms: float = -1.0):
        """Raw int16 ADC chunk; pA = (raw + offset) * range / digitisation."""
        s = np.ascontiguousarray(samples, dtype=np.int16)
        _check(self._lib.dtwx_submit_chunk_i16(self._h, channel, read_number, _ptr(s), s.size, int(is_last),
                                               float(arrival_ms), float(offset), float(range_),
                                               float(digitisation)), self._h)

    def serve_step(self) -> int:
        return _check(self._lib.dtwx_serve_step(self._h), self._h)

    def poll_decisions(self, cap: int = 4096):
        buf = getattr(self, "_dbuf", None)
        if buf is None or len(buf) < cap:
            buf = self._dbuf = (Decision * cap)()
        n = _check(self._lib.dtwx_poll_decisions(self._h, buf, cap), self._h)
        return [{f: getattr(buf[i], f) for f, _ in Decision._fields_} for i in range(n)]

    def serve_drain(self):
        _check(self._lib.dtwx_serve_drain(self._h), self._h)

    def stats(self) -> dict:
        st = Stats()
        _check(self._lib.dtwx_stats_get(self._h, ctypes.byref(st)), self._h)
        return {f: getattr(st, f) for f, _ in Stats._fields_}


def load_fasta(path: str) -> bytes:
    """Sequence of a FASTA file under the reference's single-record rules (host only)."""
    L = load_library()
    n = ctypes.c_int64()
    _check(L.dtwx_load_fasta(path.encode(), None, 0, ctypes.byref(n)))
    buf = ctypes.create_string_buffer(max(n.value, 1))
    _check(L.dtwx_load_fasta(path.encode(), buf, n.value, ctypes.byref(n)))
    return buf.raw[: n.value]


def load_kmer_model(path: str) -> np.ndarray:
    """4096 k-mer means by 2-bit code (host only)."""
    t = np.zeros(4096, np.float32)
    _check(load_library().dtwx_load_kmer_model(path.encode(), _ptr(t)))
    return t


def peak_probe(device: int = 0, precision: int = FP16, ms_target: float = 200.0) -> float:
    """Cells/s ceiling of the cell-update instruction mix on this GPU."""
    v = ctypes.c_double()
    _check(load_library().dtwx_peak_probe(device, precision, ms_target, ctypes.byref(v)))
    return v.value


def now_ms() -> float:
    return float(load_library().dtwx_now_ms())


def format_log(results: np.ndarray, read_ids: Sequence[str], ref_len: int) -> str:
    """The reference's 6-column log (src/main.cu:289-297); skipped reads are
    left out, as the reference drops reads shorter than its window."""
    lines = ["Read_ID\tQUERY_LEN\tREF_LEN\tsDTW score: fwd-strand\tsDTW score: rev-strand"]
    j = 0
    for r, rid in zip(results, read_ids):
        if r["call"] < 0:
            continue
        lines.append(f"{j}\t{rid}\t{int(r['n_samples'])}\t{ref_len}\t{float(r['score_fwd']):g}\t{float(r['score_rev']):g}")
        j += 1
    return "\n".join(lines) + "\n"
