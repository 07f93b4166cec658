"""Python mirror of the reference's pairwise API over the C ABI.

Names, fields, defaults and error behaviour follow
include/genoaligner/api.hpp of alrobles/genoaligner (AlignRequest,
AlignResult, BatchResult, align, align_batch, SWScoring, SWRequest,
SWAlignResult, SWBatchResult, align_sw, align_sw_batch, backend_name,
device_name, device_available).  Every call goes through
libgenoaligner_gb300.so (include/genoaligner_gb300.h); there is no Python or
CPU fallback: if the library is missing, importing the binding raises.

Besides the object API, ``align_batch_packed`` / ``align_sw_batch_packed``
take sequences already concatenated in one buffer (offsets + lengths), the
layout bulk callers and the benchmark hold; they build the C request arrays
with numpy and return numpy result arrays.
"""
from __future__ import annotations

import ctypes
import enum
import os
from dataclasses import dataclass, field

import numpy as np

from . import _build

GA_OK, GA_INVALID_ARGUMENT, GA_DEVICE_ERROR = 0, 1, 2
GA_MAX_SMAX, GA_MAX_SMAX_DEVICE = 511, 3500       # include/genoaligner_gb300.h
K_MAX_SMAX = 511
SW_MAX_TRACE_CELLS = 1 << 26

REQ_DT = np.dtype([("pattern", "<u8"), ("pattern_len", "<i4"), ("smax", "<i4"),
                   ("text", "<u8"), ("text_len", "<i4"), ("with_cigar", "<i4")])
RES_DT = np.dtype([("score", "<i4"), ("resolved", "<i4"), ("rescore_ok", "<i4"),
                   ("wellformed_ok", "<i4"), ("cigar_offset", "<i8"), ("cigar_len", "<i4"),
                   ("reserved", "<i4")])
SWREQ_DT = np.dtype([("text", "<u8"), ("text_len", "<i4"), ("with_cigar", "<i4"),
                     ("pattern", "<u8"), ("pattern_len", "<i4"), ("reserved", "<i4"),
                     ("match", "<i4"), ("mismatch", "<i4"), ("gap_open", "<i4"),
                     ("gap_extend", "<i4")])
SWRES_DT = np.dtype([("score", "<i4"), ("resolved", "<i4"), ("start_i", "<i4"),
                     ("start_j", "<i4"), ("end_i", "<i4"), ("end_j", "<i4"),
                     ("rescore_ok", "<i4"), ("wellformed_ok", "<i4"), ("too_large", "<i4"),
                     ("cigar_len", "<i4"), ("cigar_offset", "<i8")])
assert REQ_DT.itemsize == 32 and RES_DT.itemsize == 32
assert SWREQ_DT.itemsize == 48 and SWRES_DT.itemsize == 48


class BatchInfo(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int32), ("resolved_count", ctypes.c_int32),
                ("unresolved_count", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("error", ctypes.c_char_p)]


class Options(ctypes.Structure):
    _fields_ = [("max_smax", ctypes.c_int32), ("learned", ctypes.c_int32),
                ("trace_cell_limit", ctypes.c_int64), ("reserved", ctypes.c_int32 * 4)]


class SwScoringC(ctypes.Structure):
    _fields_ = [("match", ctypes.c_int32), ("mismatch", ctypes.c_int32),
                ("gap_open", ctypes.c_int32), ("gap_extend", ctypes.c_int32)]


class TuneC(ctypes.Structure):
    _fields_ = [("sw_pack16", ctypes.c_int32), ("sw_window", ctypes.c_int32),
                ("sw_long_log2", ctypes.c_int32), ("wfa_lane_smax", ctypes.c_int32),
                ("sw_coop_log2", ctypes.c_int32), ("sw_opt16_pct", ctypes.c_int32), ("wfa_group", ctypes.c_int32),
                ("reserved", ctypes.c_int32 * 1)]


class TuneTrialC(ctypes.Structure):
    _fields_ = [("tune", TuneC), ("ms", ctypes.c_double)]


TUNE_FIELDS = ("sw_pack16", "sw_window", "sw_long_log2", "wfa_lane_smax", "sw_coop_log2", "sw_opt16_pct",
               "wfa_group")


class DeviceBatch(ctypes.Structure):
    _fields_ = [("seq", ctypes.c_void_p), ("seq_bytes", ctypes.c_int64),
                ("a_off", ctypes.c_void_p), ("a_len", ctypes.c_void_p),
                ("b_off", ctypes.c_void_p), ("b_len", ctypes.c_void_p),
                ("out_off", ctypes.c_void_p), ("n", ctypes.c_int32), ("reserved", ctypes.c_int32)]


EXPORTS = ["ga_align_cigar_bytes", "ga_align_batch", "ga_align_sw_cigar_bytes", "ga_align_sw_batch",
           "ga_align_batch_ex", "ga_align_sw_batch_ex", "ga_wfa_device", "ga_sw_device",
           "ga_backend_name", "ga_device_name", "ga_device_available", "ga_kernel_launches",
           "ga_debug_fail_next", "ga_last_transfer_bytes", "ga_profile", "ga_profile_read",
           "ga_profile_kernel_name", "ga_bench_int_peak", "ga_cost_model_nparams", "ga_cost_model_set",
           "ga_cost_model_get", "ga_wfa_features", "ga_mlp_forward", "ga_mlp_gradient", "ga_mlp_train_step",
           "ga_wfa_device_ex", "ga_wfa_route_stats", "ga_wfa_route_items", "ga_sw_device_ex", "ga_model_select",
           "ga_sw_features", "ga_mlp_forward_fast", "ga_tune_default", "ga_tune_get",
           "ga_tune_set", "ga_autotune_sw", "ga_autotune_wfa", "ga_tune_save", "ga_tune_load",
           "ga_fasta_read", "ga_fasta_parse", "ga_fasta_count", "ga_fasta_id", "ga_fasta_description",
           "ga_fasta_arena", "ga_fasta_offsets", "ga_fasta_lengths", "ga_fasta_pinned", "ga_fasta_upload",
           "ga_fasta_free", "ga_pack_2bit_device", "ga_sw_qc_device", "ga_sw_validate_device",
           "ga_wfa_validate_device"]

_lib = None


def library_path() -> str:
    return _build.LIB


def load(build: bool = True):
    """Load (building first if needed) libgenoaligner_gb300.so."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build else _build.LIB
    if not os.path.exists(path):
        raise ImportError(f"libgenoaligner_gb300.so not built at {path}")
    L = ctypes.CDLL(path)
    p, i32, i64 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64
    L.ga_align_cigar_bytes.argtypes = [p, i32]
    L.ga_align_cigar_bytes.restype = i64
    L.ga_align_sw_cigar_bytes.argtypes = [p, i32]
    L.ga_align_sw_cigar_bytes.restype = i64
    L.ga_align_batch.argtypes = [p, i32, p, p, i64, ctypes.POINTER(BatchInfo)]
    L.ga_align_batch.restype = i32
    L.ga_align_batch_ex.argtypes = [p, i32, p, p, i64, ctypes.POINTER(Options), ctypes.POINTER(BatchInfo)]
    L.ga_align_batch_ex.restype = i32
    L.ga_align_sw_batch.argtypes = [p, i32, p, p, i64, ctypes.POINTER(BatchInfo)]
    L.ga_align_sw_batch.restype = i32
    L.ga_align_sw_batch_ex.argtypes = [p, i32, p, p, i64, ctypes.POINTER(Options), ctypes.POINTER(BatchInfo)]
    L.ga_align_sw_batch_ex.restype = i32
    L.ga_wfa_device.argtypes = [ctypes.POINTER(DeviceBatch), i32, i32, p, p, p, p, ctypes.POINTER(ctypes.c_char_p)]
    L.ga_wfa_device.restype = i32
    L.ga_sw_device.argtypes = [ctypes.POINTER(DeviceBatch), SwScoringC, i32, i64, p, p, p, p, p,
                               ctypes.POINTER(ctypes.c_char_p)]
    L.ga_sw_device.restype = i32
    L.ga_sw_device_ex.argtypes = [ctypes.POINTER(DeviceBatch), SwScoringC, i32, i64, ctypes.POINTER(Options), p, p,
                                  p, p, p, ctypes.POINTER(ctypes.c_char_p)]
    L.ga_sw_device_ex.restype = i32
    L.ga_backend_name.restype = ctypes.c_char_p
    L.ga_device_name.restype = ctypes.c_char_p
    L.ga_device_available.restype = i32
    L.ga_kernel_launches.restype = i64
    L.ga_debug_fail_next.argtypes = [i32]
    L.ga_last_transfer_bytes.argtypes = [ctypes.POINTER(i64), ctypes.POINTER(i64)]
    L.ga_profile.argtypes = [i32]
    L.ga_profile_read.argtypes = [i32, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(i64)]
    L.ga_profile_read.restype = i32
    L.ga_profile_kernel_name.argtypes = [i32]
    L.ga_profile_kernel_name.restype = ctypes.c_char_p
    L.ga_bench_int_peak.argtypes = [i32, ctypes.POINTER(ctypes.c_double)]
    L.ga_bench_int_peak.restype = i32
    L.ga_cost_model_nparams.restype = i32
    L.ga_cost_model_set.argtypes = [p, i32]
    L.ga_cost_model_set.restype = i32
    L.ga_cost_model_get.argtypes = [p, i32]
    L.ga_cost_model_get.restype = i32
    L.ga_wfa_features.argtypes = [ctypes.POINTER(DeviceBatch), p, p, p]
    L.ga_wfa_features.restype = i32
    L.ga_mlp_forward.argtypes = [p, i32, p, p]
    L.ga_mlp_forward.restype = i32
    L.ga_mlp_gradient.argtypes = [p, p, i32, p, p]
    L.ga_mlp_gradient.restype = i32
    L.ga_mlp_train_step.argtypes = [p, p, i32, ctypes.c_float, p, p]
    L.ga_mlp_train_step.restype = i32
    L.ga_wfa_device_ex.argtypes = [ctypes.POINTER(DeviceBatch), i32, i32, ctypes.POINTER(Options), p, p, p, p,
                                   ctypes.POINTER(ctypes.c_char_p)]
    L.ga_wfa_device_ex.restype = i32
    L.ga_mlp_forward_fast.argtypes = [p, i32, p, p]
    L.ga_mlp_forward_fast.restype = i32
    L.ga_wfa_route_stats.argtypes = [p, i32]
    L.ga_wfa_route_stats.restype = i32
    L.ga_wfa_route_items.argtypes = [p, i32]
    L.ga_wfa_route_items.restype = i32
    L.ga_model_select.argtypes = [i32]
    L.ga_model_select.restype = i32
    L.ga_sw_features.argtypes = [ctypes.POINTER(DeviceBatch), p, p]
    L.ga_sw_features.restype = i32
    for f in ("ga_tune_default", "ga_tune_get"):
        getattr(L, f).argtypes = [ctypes.POINTER(TuneC)]
        getattr(L, f).restype = i32
    L.ga_tune_set.argtypes = [ctypes.POINTER(TuneC)]
    L.ga_tune_set.restype = i32
    L.ga_autotune_sw.argtypes = [ctypes.POINTER(DeviceBatch), SwScoringC, i64, p, p, p, p, i32,
                                 ctypes.POINTER(TuneC), p, i32, ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_char_p)]
    L.ga_autotune_sw.restype = i32
    L.ga_autotune_wfa.argtypes = [ctypes.POINTER(DeviceBatch), i32, i32, p, p, p, i32,
                                  ctypes.POINTER(TuneC), p, i32, ctypes.POINTER(i32), ctypes.POINTER(ctypes.c_char_p)]
    L.ga_autotune_wfa.restype = i32
    L.ga_tune_save.argtypes = [ctypes.c_char_p]
    L.ga_tune_save.restype = i32
    L.ga_tune_load.argtypes = [ctypes.c_char_p]
    L.ga_tune_load.restype = i32
    pp = ctypes.POINTER(ctypes.c_void_p)
    L.ga_fasta_read.argtypes = [ctypes.c_char_p, pp, ctypes.POINTER(ctypes.c_char_p)]
    L.ga_fasta_read.restype = i32
    L.ga_fasta_parse.argtypes = [ctypes.c_char_p, i64, pp, ctypes.POINTER(ctypes.c_char_p)]
    L.ga_fasta_parse.restype = i32
    L.ga_fasta_count.argtypes = [p]
    L.ga_fasta_count.restype = i32
    for f in ("ga_fasta_id", "ga_fasta_description"):
        getattr(L, f).argtypes = [p, i32]
        getattr(L, f).restype = ctypes.c_char_p
    L.ga_fasta_arena.argtypes = [p, ctypes.POINTER(i64)]
    L.ga_fasta_arena.restype = p
    L.ga_fasta_offsets.argtypes = [p]
    L.ga_fasta_offsets.restype = p
    L.ga_fasta_lengths.argtypes = [p]
    L.ga_fasta_lengths.restype = p
    L.ga_fasta_pinned.argtypes = [p]
    L.ga_fasta_pinned.restype = i32
    L.ga_fasta_upload.argtypes = [p, p, p]
    L.ga_fasta_upload.restype = i32
    L.ga_fasta_free.argtypes = [p]
    L.ga_fasta_free.restype = None
    L.ga_pack_2bit_device.argtypes = [p, i64, p, p, p]
    L.ga_pack_2bit_device.restype = i32
    L.ga_sw_qc_device.argtypes = [ctypes.POINTER(DeviceBatch), p, p, p, p, i32, i32, p, p]
    L.ga_sw_qc_device.restype = i32
    L.ga_sw_validate_device.argtypes = [ctypes.POINTER(DeviceBatch), SwScoringC, p, p, p, p, p, p]
    L.ga_sw_validate_device.restype = i32
    L.ga_wfa_validate_device.argtypes = [ctypes.POINTER(DeviceBatch), p, p, p, p, p]
    L.ga_wfa_validate_device.restype = i32
    _lib = L
    return L


# ----------------------------------------------------------------- types --
class Status(enum.Enum):
    ok = 0
    invalid_argument = 1
    device_error = 2


@dataclass
class AlignRequest:
    pattern: bytes | None = None
    pattern_len: int = 0
    text: bytes | None = None
    text_len: int = 0
    smax: int = 64
    with_cigar: bool = True


@dataclass
class AlignResult:
    score: int = -1
    resolved: bool = False
    cigar: str = ""
    rescore_ok: bool = False
    wellformed_ok: bool = False


@dataclass
class BatchResult:
    results: list = field(default_factory=list)
    resolved_count: int = 0
    unresolved_count: int = 0
    status: Status = Status.ok
    error: str | None = None

    def ok(self) -> bool:
        return self.status == Status.ok


@dataclass
class SWScoring:
    match: int = 2
    mismatch: int = -3
    gap_open: int = 5
    gap_extend: int = 2


@dataclass
class SWRequest:
    text: bytes | None = None
    text_len: int = 0
    pattern: bytes | None = None
    pattern_len: int = 0
    scoring: SWScoring = field(default_factory=SWScoring)
    with_cigar: bool = True


@dataclass
class SWAlignResult:
    score: int = -1
    resolved: bool = False
    cigar: str = ""
    start_i: int = -1
    start_j: int = -1
    end_i: int = -1
    end_j: int = -1
    rescore_ok: bool = False
    wellformed_ok: bool = False
    too_large: bool = False


@dataclass
class SWBatchResult:
    results: list = field(default_factory=list)
    resolved_count: int = 0
    unresolved_count: int = 0
    status: Status = Status.ok
    error: str | None = None

    def ok(self) -> bool:
        return self.status == Status.ok


def _addr(b):
    """Address of a bytes object's buffer (None -> 0)."""
    if b is None:
        return 0
    return ctypes.cast(ctypes.c_char_p(b), ctypes.c_void_p).value or 0


def _opts(max_smax=0, learned=False, trace_cell_limit=0):
    o = Options()
    o.max_smax = max_smax
    # True / 1: queues by the cost model; 2: the same queues by the exact
    # lower bound alone (no network)
    o.learned = 2 if (learned == 2 and learned is not True) else (1 if learned else 0)
    o.trace_cell_limit = trace_cell_limit
    return o


def align_batch(reqs, max_smax: int = 0, learned: bool = False) -> BatchResult:
    """genoaligner::align_batch (or align_batch_ex with max_smax / learned)."""
    L = load()
    n = len(reqs)
    if n == 0:
        return BatchResult()
    keep = []
    arr = np.zeros(n, REQ_DT)
    for i, r in enumerate(reqs):
        keep.append(r.pattern)
        keep.append(r.text)
        arr[i] = (_addr(r.pattern), r.pattern_len, r.smax, _addr(r.text), r.text_len, 1 if r.with_cigar else 0)
    res = np.zeros(n, RES_DT)
    nbytes = int(L.ga_align_cigar_bytes(arr.ctypes.data, n))
    buf = ctypes.create_string_buffer(max(nbytes, 1))
    info = BatchInfo()
    if max_smax or learned:
        o = _opts(max_smax, learned)
        st = L.ga_align_batch_ex(arr.ctypes.data, n, res.ctypes.data, buf, nbytes, ctypes.byref(o), ctypes.byref(info))
    else:
        st = L.ga_align_batch(arr.ctypes.data, n, res.ctypes.data, buf, nbytes, ctypes.byref(info))
    out = BatchResult(status=Status(st), error=info.error.decode() if info.error else None,
                      resolved_count=info.resolved_count, unresolved_count=info.unresolved_count)
    raw = buf.raw
    for i in range(n):
        r = res[i]
        off, ln = int(r["cigar_offset"]), int(r["cigar_len"])
        out.results.append(AlignResult(int(r["score"]), bool(r["resolved"]),
                                       raw[off:off + ln].decode("latin-1") if ln else "",
                                       bool(r["rescore_ok"]), bool(r["wellformed_ok"])))
    return out


def align(req: AlignRequest) -> AlignResult:
    b = align_batch([req])
    return b.results[0] if b.results else AlignResult()


def align_sw_batch(reqs, trace_cell_limit: int = 0, learned: bool = False) -> SWBatchResult:
    """genoaligner::align_sw_batch (or align_sw_batch_ex with a trace limit, < 0 = none,
    or with the SW variant model's routing)."""
    L = load()
    n = len(reqs)
    if n == 0:
        return SWBatchResult()
    keep = []
    arr = np.zeros(n, SWREQ_DT)
    for i, r in enumerate(reqs):
        keep.append(r.text)
        keep.append(r.pattern)
        s = r.scoring
        arr[i] = (_addr(r.text), r.text_len, 1 if r.with_cigar else 0, _addr(r.pattern), r.pattern_len, 0,
                  s.match, s.mismatch, s.gap_open, s.gap_extend)
    res = np.zeros(n, SWRES_DT)
    nbytes = int(L.ga_align_sw_cigar_bytes(arr.ctypes.data, n))
    buf = ctypes.create_string_buffer(max(nbytes, 1))
    info = BatchInfo()
    if trace_cell_limit or learned:
        o = _opts(learned=learned, trace_cell_limit=trace_cell_limit)
        st = L.ga_align_sw_batch_ex(arr.ctypes.data, n, res.ctypes.data, buf, nbytes, ctypes.byref(o),
                                    ctypes.byref(info))
    else:
        st = L.ga_align_sw_batch(arr.ctypes.data, n, res.ctypes.data, buf, nbytes, ctypes.byref(info))
    out = SWBatchResult(status=Status(st), error=info.error.decode() if info.error else None,
                        resolved_count=info.resolved_count, unresolved_count=info.unresolved_count)
    raw = buf.raw
    for i in range(n):
        r = res[i]
        off, ln = int(r["cigar_offset"]), int(r["cigar_len"])
        out.results.append(SWAlignResult(int(r["score"]), bool(r["resolved"]),
                                         raw[off:off + ln].decode("latin-1") if ln else "",
                                         int(r["start_i"]), int(r["start_j"]), int(r["end_i"]),
                                         int(r["end_j"]), bool(r["rescore_ok"]), bool(r["wellformed_ok"]),
                                         bool(r["too_large"])))
    return out


def align_sw(req: SWRequest) -> SWAlignResult:
    b = align_sw_batch([req])
    return b.results[0] if b.results else SWAlignResult()


def backend_name() -> str:
    return load().ga_backend_name().decode()


def device_name() -> str:
    return load().ga_device_name().decode()


def device_available() -> bool:
    return bool(load().ga_device_available())


def kernel_launches() -> int:
    return int(load().ga_kernel_launches())


def last_transfer_bytes():
    h, d = ctypes.c_int64(0), ctypes.c_int64(0)
    load().ga_last_transfer_bytes(ctypes.byref(h), ctypes.byref(d))
    return int(h.value), int(d.value)


def profile(on: bool):
    load().ga_profile(1 if on else 0)


def profile_read():
    """{kernel name: (total device ms, launches)} for kernels that ran."""
    L = load()
    out = {}
    for k in range(64):
        name = L.ga_profile_kernel_name(k)
        if not name:
            break
        name = name.decode()
        ms, n = ctypes.c_double(0), ctypes.c_int64(0)
        L.ga_profile_read(k, ctypes.byref(ms), ctypes.byref(n))
        if n.value:
            out[name] = (float(ms.value), int(n.value))
    return out


def int_peak(variant: int = 0) -> float:
    v = ctypes.c_double(0)
    st = load().ga_bench_int_peak(variant, ctypes.byref(v))
    if st != GA_OK:
        raise RuntimeError("int peak microbenchmark failed")
    return float(v.value)


# -------------------------------------------------------- device-resident --
def device_layout(a_buf, a_off, a_len, b_buf, b_off, b_len):
    """Host-side plan of the device arena: every sequence at a 32-byte-aligned
    offset, 64 bytes of padding at the end, CIGAR slots of a_len + b_len.
    Returns (arena uint8, a_off, b_off, out_off, out_bytes)."""
    n = a_len.shape[0]
    ra = (a_len.astype(np.int64) + 31) & ~31
    rb = (b_len.astype(np.int64) + 31) & ~31
    step = ra + rb
    base = np.zeros(n, np.int64)
    if n > 1:
        np.cumsum(step[:-1], out=base[1:])
    na_off = base
    nb_off = base + ra
    total = int(step.sum()) + 64
    arena = np.zeros(total, np.uint8)
    _scatter(arena, na_off, a_buf, a_off, a_len)
    _scatter(arena, nb_off, b_buf, b_off, b_len)
    cap = a_len.astype(np.int64) + b_len
    out_off = np.zeros(n, np.int64)
    if n > 1:
        np.cumsum(cap[:-1], out=out_off[1:])
    return arena, na_off, nb_off, out_off, int(cap.sum())


def _scatter(dst, dst_off, src, src_off, lens):
    lens64 = lens.astype(np.int64)
    tot = int(lens64.sum())
    if tot == 0:
        return
    seg = np.repeat(np.arange(lens.shape[0]), lens64)
    starts = np.zeros(lens.shape[0], np.int64)
    if lens.shape[0] > 1:
        np.cumsum(lens64[:-1], out=starts[1:])
    within = np.arange(tot, dtype=np.int64) - starts[seg]
    dst[dst_off[seg] + within] = src[src_off[seg] + within]


class DeviceBatchT:
    """A batch resident in device memory (torch tensors) for ga_wfa_device /
    ga_sw_device."""

    def __init__(self, a_buf, a_off, a_len, b_buf, b_off, b_len, device="cuda:0"):
        import torch
        arena, na, nb, oo, out_bytes = device_layout(a_buf, a_off, a_len, b_buf, b_off, b_len)
        self.n = int(a_len.shape[0])
        self.seq = torch.from_numpy(arena).to(device)
        self.a_off = torch.from_numpy(na).to(device)
        self.a_len = torch.from_numpy(a_len.astype(np.int32)).to(device)
        self.b_off = torch.from_numpy(nb).to(device)
        self.b_len = torch.from_numpy(b_len.astype(np.int32)).to(device)
        self.out_off = torch.from_numpy(oo).to(device)
        self.out_bytes = out_bytes
        self.input_bytes = int(arena.nbytes + 8 * 3 * self.n + 4 * 2 * self.n)
        self.c = DeviceBatch(self.seq.data_ptr(), int(arena.shape[0]), self.a_off.data_ptr(),
                             self.a_len.data_ptr(), self.b_off.data_ptr(), self.b_len.data_ptr(),
                             self.out_off.data_ptr(), self.n, 0)

    @classmethod
    def from_device_arena(cls, seq, a_off, a_len, b_off, b_len):
        """A batch over a byte arena already in device memory (a uint8 tensor,
        sequences at 32-byte-aligned offsets, 64 spare bytes at the end): numpy
        offsets and lengths; CIGAR slots of a_len + b_len bytes in pair order."""
        import torch
        self = cls.__new__(cls)
        dev = seq.device
        a_len = np.asarray(a_len, np.int32)
        b_len = np.asarray(b_len, np.int32)
        self.n = int(a_len.shape[0])
        cap = a_len.astype(np.int64) + b_len
        oo = np.zeros(self.n, np.int64)
        if self.n:
            oo[1:] = np.cumsum(cap)[:-1]
        self.seq = seq
        self.a_off = torch.from_numpy(np.ascontiguousarray(a_off, np.int64)).to(dev)
        self.a_len = torch.from_numpy(a_len).to(dev)
        self.b_off = torch.from_numpy(np.ascontiguousarray(b_off, np.int64)).to(dev)
        self.b_len = torch.from_numpy(b_len).to(dev)
        self.out_off = torch.from_numpy(oo).to(dev)
        self.out_bytes = int(cap.sum())
        self.input_bytes = int(seq.numel() + 8 * 3 * self.n + 4 * 2 * self.n)
        self.c = DeviceBatch(seq.data_ptr(), int(seq.numel()), self.a_off.data_ptr(), self.a_len.data_ptr(),
                             self.b_off.data_ptr(), self.b_len.data_ptr(), self.out_off.data_ptr(), self.n, 0)
        return self


def wfa_device(batch: DeviceBatchT, smax, trace, out_score, out_len, out_cigar, stream=None, learned=False):
    err = ctypes.c_char_p()
    o = _opts(0, learned)
    st = load().ga_wfa_device_ex(ctypes.byref(batch.c), smax, 1 if trace else 0, ctypes.byref(o),
                                 out_score.data_ptr(),
                                 out_len.data_ptr() if out_len is not None else None,
                                 out_cigar.data_ptr() if out_cigar is not None else None,
                                 stream, ctypes.byref(err))
    if st != GA_OK:
        raise RuntimeError(f"ga_wfa_device failed: {err.value}")


def sw_device(batch: DeviceBatchT, scoring, trace, out_score, out_pos, out_len, out_cigar, stream=None,
              trace_cell_limit=-1, learned=False):
    """ga_sw_device, or ga_sw_device_ex with learned = 1 (the SW variant
    model routes pairs to the 16-bit kernel)."""
    err = ctypes.c_char_p()
    sc = SwScoringC(*scoring)
    L = load()
    args = (out_score.data_ptr(), out_pos.data_ptr(), out_len.data_ptr() if out_len is not None else None,
            out_cigar.data_ptr() if out_cigar is not None else None, stream, ctypes.byref(err))
    if learned:
        o = _opts(learned=True)
        st = L.ga_sw_device_ex(ctypes.byref(batch.c), sc, 1 if trace else 0, trace_cell_limit, ctypes.byref(o), *args)
    else:
        st = L.ga_sw_device(ctypes.byref(batch.c), sc, 1 if trace else 0, trace_cell_limit, *args)
    if st != GA_OK:
        raise RuntimeError(f"ga_sw_device failed: {err.value}")


# ------------------------------------------------------------ packed bulk --
@dataclass
class PackedResult:
    """Result arrays of a packed batch call; CIGAR i = cigar_buf[off[i]:off[i]+len[i]]."""
    status: Status
    error: str | None
    res: np.ndarray
    cigar_buf: np.ndarray
    resolved_count: int
    unresolved_count: int

    def cigar(self, i: int) -> bytes:
        o, ln = int(self.res["cigar_offset"][i]), int(self.res["cigar_len"][i])
        return self.cigar_buf[o:o + ln].tobytes()


def align_batch_packed(p_buf, p_off, p_len, t_buf, t_off, t_len, smax=64, with_cigar=True,
                       max_smax=0, learned=False, _reqs=None, _res=None, _cig=None) -> PackedResult:
    """align_batch over sequences held in two byte buffers (pattern i =
    p_buf[p_off[i]:p_off[i]+p_len[i]], text likewise).  ``smax`` and
    ``with_cigar`` are scalars or per-request arrays.  The optional ``_reqs``,
    ``_res``, ``_cig`` let a caller reuse its request/result/CIGAR arrays."""
    L = load()
    n = int(p_len.shape[0])
    reqs = _reqs if _reqs is not None else make_requests(p_buf, p_off, p_len, t_buf, t_off, t_len, smax, with_cigar)
    res = _res if _res is not None else np.zeros(n, RES_DT)
    nbytes = int(L.ga_align_cigar_bytes(reqs.ctypes.data, n))
    cig = _cig if _cig is not None and _cig.shape[0] >= nbytes else np.empty(max(nbytes, 1), np.uint8)
    info = BatchInfo()
    if max_smax or learned:
        o = _opts(max_smax, learned)
        st = L.ga_align_batch_ex(reqs.ctypes.data, n, res.ctypes.data, cig.ctypes.data, nbytes,
                                 ctypes.byref(o), ctypes.byref(info))
    else:
        st = L.ga_align_batch(reqs.ctypes.data, n, res.ctypes.data, cig.ctypes.data, nbytes, ctypes.byref(info))
    return PackedResult(Status(st), info.error.decode() if info.error else None, res, cig,
                        info.resolved_count, info.unresolved_count)


def make_requests(p_buf, p_off, p_len, t_buf, t_off, t_len, smax=64, with_cigar=True) -> np.ndarray:
    n = int(p_len.shape[0])
    reqs = np.zeros(n, REQ_DT)
    reqs["pattern"] = p_buf.ctypes.data + p_off.astype(np.uint64)
    reqs["pattern_len"] = p_len
    reqs["smax"] = smax
    reqs["text"] = t_buf.ctypes.data + t_off.astype(np.uint64)
    reqs["text_len"] = t_len
    reqs["with_cigar"] = np.asarray(with_cigar).astype(np.int32)
    return reqs


def make_sw_requests(t_buf, t_off, t_len, p_buf, p_off, p_len, scoring=(2, -3, 5, 2), with_cigar=True) -> np.ndarray:
    n = int(t_len.shape[0])
    reqs = np.zeros(n, SWREQ_DT)
    reqs["text"] = t_buf.ctypes.data + t_off.astype(np.uint64)
    reqs["text_len"] = t_len
    reqs["with_cigar"] = np.asarray(with_cigar).astype(np.int32)
    reqs["pattern"] = p_buf.ctypes.data + p_off.astype(np.uint64)
    reqs["pattern_len"] = p_len
    reqs["match"], reqs["mismatch"], reqs["gap_open"], reqs["gap_extend"] = scoring
    return reqs


def align_sw_batch_packed(t_buf, t_off, t_len, p_buf, p_off, p_len, scoring=(2, -3, 5, 2), with_cigar=True,
                          trace_cell_limit=0, learned=False, _reqs=None, _res=None, _cig=None) -> PackedResult:
    """align_sw_batch over packed sequences (text = rows, pattern = columns)."""
    L = load()
    n = int(t_len.shape[0])
    reqs = _reqs if _reqs is not None else make_sw_requests(t_buf, t_off, t_len, p_buf, p_off, p_len, scoring,
                                                            with_cigar)
    res = _res if _res is not None else np.zeros(n, SWRES_DT)
    if _cig is not None:                      # a caller's buffer: the library checks its size
        cig, nbytes = _cig, int(_cig.shape[0])
    else:
        nbytes = int(L.ga_align_sw_cigar_bytes(reqs.ctypes.data, n))
        cig = np.empty(max(nbytes, 1), np.uint8)
    info = BatchInfo()
    if trace_cell_limit or learned:
        o = _opts(learned=learned, trace_cell_limit=trace_cell_limit)
        st = L.ga_align_sw_batch_ex(reqs.ctypes.data, n, res.ctypes.data, cig.ctypes.data, nbytes,
                                    ctypes.byref(o), ctypes.byref(info))
    else:
        st = L.ga_align_sw_batch(reqs.ctypes.data, n, res.ctypes.data, cig.ctypes.data, nbytes, ctypes.byref(info))
    return PackedResult(Status(st), info.error.decode() if info.error else None, res, cig,
                        info.resolved_count, info.unresolved_count)


# ---------------------------------------------------------- learned model --
def cost_model_nparams() -> int:
    return int(load().ga_cost_model_nparams())


def cost_model_set(params: np.ndarray):
    p = np.ascontiguousarray(params, dtype=np.float32)
    st = load().ga_cost_model_set(p.ctypes.data, int(p.shape[0]))
    if st != GA_OK:
        raise RuntimeError(f"ga_cost_model_set failed ({st})")


def cost_model_get() -> np.ndarray:
    p = np.zeros(cost_model_nparams(), np.float32)
    st = load().ga_cost_model_get(p.ctypes.data, int(p.shape[0]))
    if st != GA_OK:
        raise RuntimeError(f"ga_cost_model_get failed ({st})")
    return p


def cost_model_init(seed: int = 0) -> np.ndarray:
    """He-initialised parameters in the library's layout."""
    rng = np.random.default_rng(seed)
    parts = []
    for fan_in, fan_out in ((66, 128), (128, 128), (128, 2)):
        parts.append(rng.normal(0, np.sqrt(2.0 / fan_in), size=fan_out * fan_in).astype(np.float32))
        parts.append(np.zeros(fan_out, np.float32))
    return np.concatenate(parts)


def model_select(which: int):
    """The model slot the calling thread's cost_model_* / mlp_* calls act on:
    0 the WFA cost model, 1 the SW variant model."""
    if load().ga_model_select(int(which)) != GA_OK:
        raise ValueError(f"no model slot {which}")


class model_slot:
    """with model_slot(1): ... -- select a slot, then slot 0 again."""

    def __init__(self, which: int):
        self.which = which

    def __enter__(self):
        model_select(self.which)
        return self

    def __exit__(self, *exc):
        model_select(0)
        return False


def sw_features(batch: "DeviceBatchT"):
    """Features [n,66] of an SW batch for the SW variant model (torch, on the batch's device)."""
    import torch
    feat = torch.empty((batch.n, 66), dtype=torch.float32, device=batch.seq.device)
    st = load().ga_sw_features(ctypes.byref(batch.c), feat.data_ptr(), None)
    if st != GA_OK:
        raise RuntimeError(f"ga_sw_features failed ({st})")
    return feat


def wfa_features(batch: "DeviceBatchT"):
    """(features [n,66] float32, lower bound [n] int32) as torch tensors on the batch's device."""
    import torch
    dev = batch.seq.device
    feat = torch.empty((batch.n, 66), dtype=torch.float32, device=dev)
    lb = torch.empty(batch.n, dtype=torch.int32, device=dev)
    st = load().ga_wfa_features(ctypes.byref(batch.c), feat.data_ptr(), lb.data_ptr(), None)
    if st != GA_OK:
        raise RuntimeError(f"ga_wfa_features failed ({st})")
    return feat, lb


def mlp_forward(feat):
    import torch
    y = torch.empty((feat.shape[0], 2), dtype=torch.float32, device=feat.device)
    st = load().ga_mlp_forward(feat.data_ptr(), int(feat.shape[0]), y.data_ptr(), None)
    if st != GA_OK:
        raise RuntimeError(f"ga_mlp_forward failed ({st})")
    return y


def mlp_forward_fast(feat):
    """The tensor-core routing forward pass."""
    import torch
    y = torch.empty((feat.shape[0], 2), dtype=torch.float32, device=feat.device)
    st = load().ga_mlp_forward_fast(feat.data_ptr(), int(feat.shape[0]), y.data_ptr(), None)
    if st != GA_OK:
        raise RuntimeError(f"ga_mlp_forward_fast failed ({st})")
    return y


def mlp_gradient(feat, target):
    g = np.zeros(cost_model_nparams(), np.float32)
    loss = np.zeros(1, np.float32)
    st = load().ga_mlp_gradient(feat.data_ptr(), target.data_ptr(), int(feat.shape[0]), g.ctypes.data,
                                loss.ctypes.data)
    if st != GA_OK:
        raise RuntimeError(f"ga_mlp_gradient failed ({st})")
    return g, float(loss[0])


def mlp_train_step(feat, target, lr: float) -> float:
    loss = np.zeros(1, np.float32)
    st = load().ga_mlp_train_step(feat.data_ptr(), target.data_ptr(), int(feat.shape[0]), ctypes.c_float(lr),
                                  loss.ctypes.data, None)
    if st != GA_OK:
        raise RuntimeError(f"ga_mlp_train_step failed ({st})")
    return float(loss[0])


def wfa_route_stats(rounds: int = 12):
    """(lane-queue pairs, warp-queue pairs, [pairs escalated from the lane queue
    to the warp queue, warp-queue pairs run on whole blocks, 0, ...]) of the
    calling thread's last learned call."""
    out = np.zeros(2 + rounds, np.int32)
    st = load().ga_wfa_route_stats(out.ctypes.data, int(out.shape[0]))
    if st != GA_OK:
        raise RuntimeError(f"ga_wfa_route_stats failed ({st})")
    return int(out[0]), int(out[1]), [int(x) for x in out[2:]]


def wfa_route_items(n: int) -> np.ndarray:
    """Queue item of every pair of the calling thread's last learned call
    (ga_wfa_route_items): -1 unresolved by the bound; else bucket | first smax << 8."""
    out = np.zeros(n, np.int32)
    st = load().ga_wfa_route_items(out.ctypes.data, int(n))
    if st != GA_OK:
        raise RuntimeError(f"ga_wfa_route_items failed ({st})")
    return out


# -------------------------------------------------------------- autotuner --
def _tune_dict(t: TuneC) -> dict:
    return {f: int(getattr(t, f)) for f in TUNE_FIELDS}


def tune_default() -> dict:
    """The built-in kernel setting (ga_tune_default)."""
    t = TuneC()
    load().ga_tune_default(ctypes.byref(t))
    return _tune_dict(t)


def tune_get() -> dict:
    """The current device's kernel setting (ga_tune_get)."""
    t = TuneC()
    load().ga_tune_get(ctypes.byref(t))
    return _tune_dict(t)


def tune_set(**fields):
    """Replace fields of the current device's setting (ga_tune_set); raises
    ValueError for values out of range."""
    cur = tune_get()
    for k, v in fields.items():
        if k not in TUNE_FIELDS:
            raise ValueError(f"unknown tune field {k}")
        cur[k] = int(v)
    t = TuneC(*[cur[f] for f in TUNE_FIELDS])
    st = load().ga_tune_set(ctypes.byref(t))
    if st != GA_OK:
        raise ValueError(f"ga_tune_set refused {cur}")


def _trials(buf, n):
    return [(_tune_dict(buf[i].tune), float(buf[i].ms)) for i in range(n)]


def autotune_sw(batch: "DeviceBatchT", scoring, out_score, out_pos, out_len, out_cigar, reps: int = 2,
                trace_cell_limit: int = -1):
    """Time candidate settings on an SW traceback batch and keep the fastest for
    the current device (ga_autotune_sw).  Returns (chosen, [(setting, ms)])."""
    t = TuneC()
    buf = (TuneTrialC * 32)()
    nt = ctypes.c_int32(0)
    err = ctypes.c_char_p()
    st = load().ga_autotune_sw(ctypes.byref(batch.c), SwScoringC(*scoring), trace_cell_limit,
                               out_score.data_ptr(), out_pos.data_ptr(), out_len.data_ptr(), out_cigar.data_ptr(),
                               reps, ctypes.byref(t), ctypes.cast(buf, ctypes.c_void_p), 32, ctypes.byref(nt),
                               ctypes.byref(err))
    if st != GA_OK:
        raise RuntimeError(f"ga_autotune_sw failed: {err.value}")
    return _tune_dict(t), _trials(buf, nt.value)


def autotune_wfa(batch: "DeviceBatchT", smax, trace, out_score, out_len, out_cigar, reps: int = 2):
    """The same for the learned WFA path (ga_autotune_wfa; the cost model must be
    loaded)."""
    t = TuneC()
    buf = (TuneTrialC * 32)()
    nt = ctypes.c_int32(0)
    err = ctypes.c_char_p()
    st = load().ga_autotune_wfa(ctypes.byref(batch.c), smax, 1 if trace else 0, out_score.data_ptr(),
                                out_len.data_ptr() if out_len is not None else None,
                                out_cigar.data_ptr() if out_cigar is not None else None,
                                reps, ctypes.byref(t), ctypes.cast(buf, ctypes.c_void_p), 32, ctypes.byref(nt),
                                ctypes.byref(err))
    if st != GA_OK:
        raise RuntimeError(f"ga_autotune_wfa failed: {err.value}")
    return _tune_dict(t), _trials(buf, nt.value)


def tune_save(path: str):
    if load().ga_tune_save(path.encode()) != GA_OK:
        raise OSError(f"ga_tune_save failed for {path}")


def tune_load(path: str):
    if load().ga_tune_load(path.encode()) != GA_OK:
        raise ValueError(f"ga_tune_load refused {path}")


# ----------------------------------------------------------------- ingest --
class FastaSet:
    """A FASTA file parsed into one device-ready arena (ga_fasta_*): ids,
    descriptions, and per record an offset (multiple of 32) and a length into
    `arena` (a numpy view of the library's pinned host buffer, valid while this
    object lives)."""

    def __init__(self, handle):
        L = load()
        self._h = handle
        n = L.ga_fasta_count(handle)
        self.n = n
        self.ids = [L.ga_fasta_id(handle, i).decode("latin-1") for i in range(n)]
        self.descriptions = [L.ga_fasta_description(handle, i).decode("latin-1") for i in range(n)]
        nb = ctypes.c_int64(0)
        ptr = L.ga_fasta_arena(handle, ctypes.byref(nb))
        self.arena = np.ctypeslib.as_array((ctypes.c_uint8 * nb.value).from_address(ptr))
        self.offsets = np.ctypeslib.as_array((ctypes.c_int64 * n).from_address(L.ga_fasta_offsets(handle))) \
            if n else np.zeros(0, np.int64)
        self.lengths = np.ctypeslib.as_array((ctypes.c_int32 * n).from_address(L.ga_fasta_lengths(handle))) \
            if n else np.zeros(0, np.int32)
        self.pinned = bool(L.ga_fasta_pinned(handle))

    def sequence(self, i: int) -> bytes:
        o, n = int(self.offsets[i]), int(self.lengths[i])
        return self.arena[o:o + n].tobytes()

    def upload(self, device_tensor, stream=None):
        """Copy the arena into a device tensor of at least arena.nbytes bytes."""
        if device_tensor.numel() * device_tensor.element_size() < self.arena.nbytes:
            raise ValueError("device buffer smaller than the arena")
        if load().ga_fasta_upload(self._h, device_tensor.data_ptr(), stream) != GA_OK:
            raise RuntimeError("ga_fasta_upload failed")

    def close(self):
        if self._h:
            self.arena = self.offsets = self.lengths = None
            load().ga_fasta_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _fasta_open(call):
    h = ctypes.c_void_p()
    err = ctypes.c_char_p()
    st = call(ctypes.byref(h), ctypes.byref(err))
    if st != GA_OK:
        raise ValueError(err.value.decode() if err.value else f"status {st}")
    return FastaSet(h.value)


def fasta_read(path: str) -> FastaSet:
    """Read a FASTA file into a pinned, device-ready arena (ga_fasta_read);
    raises ValueError with the reader's message on a malformed file."""
    return _fasta_open(lambda h, e: load().ga_fasta_read(path.encode(), h, e))


def fasta_parse(data: bytes) -> FastaSet:
    """The same from bytes in memory (ga_fasta_parse)."""
    return _fasta_open(lambda h, e: load().ga_fasta_parse(data, len(data), h, e))


def pack_2bit_device(seq, packed, mask, stream=None):
    """2-bit codes and non-ACGT masks of a device byte arena (ga_pack_2bit_device):
    seq uint8 (length a multiple of 32), packed int64 and mask int32 tensors of
    len(seq) // 32 elements."""
    st = load().ga_pack_2bit_device(seq.data_ptr(), int(seq.numel()), packed.data_ptr(), mask.data_ptr(), stream)
    if st != GA_OK:
        raise RuntimeError(f"ga_pack_2bit_device failed ({st})")


def sw_validate_device(batch: "DeviceBatchT", scoring, out_score, out_pos, out_len, out_cigar, flags, stream=None):
    """rescore_ok | wellformed_ok << 1 per pair into the uint8 device tensor
    `flags` (ga_sw_validate_device), from ga_sw_device's outputs."""
    st = load().ga_sw_validate_device(ctypes.byref(batch.c), SwScoringC(*scoring), out_score.data_ptr(),
                                      out_pos.data_ptr(), out_len.data_ptr(), out_cigar.data_ptr(), flags.data_ptr(),
                                      stream)
    if st != GA_OK:
        raise RuntimeError(f"ga_sw_validate_device failed ({st})")


def sw_qc_device(batch: "DeviceBatchT", out_score, out_pos, out_len, out_cigar, frame: int, code: int, out,
                 stream=None):
    """Per pair (fs_runs, fs_net, stops, stop_end) into the int32 device tensor
    `out` of 4 n elements (ga_sw_qc_device)."""
    st = load().ga_sw_qc_device(ctypes.byref(batch.c), out_score.data_ptr(), out_pos.data_ptr(), out_len.data_ptr(),
                                out_cigar.data_ptr(), int(frame), int(code), out.data_ptr(), stream)
    if st != GA_OK:
        raise RuntimeError(f"ga_sw_qc_device failed ({st})")


def wfa_validate_device(batch: "DeviceBatchT", out_score, out_len, out_cigar, flags, stream=None):
    """rescore_ok | wellformed_ok << 1 per pair into the uint8 device tensor
    `flags` (ga_wfa_validate_device), from ga_wfa_device's outputs."""
    st = load().ga_wfa_validate_device(ctypes.byref(batch.c), out_score.data_ptr(), out_len.data_ptr(),
                                       out_cigar.data_ptr(), flags.data_ptr(), stream)
    if st != GA_OK:
        raise RuntimeError(f"ga_wfa_validate_device failed ({st})")
