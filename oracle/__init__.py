"""CPU oracle for batched pairwise alignment -- TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import
this package, and only as the checker.  The product (genoaligner_gb300) never
imports it.

Two layers:

* ``oracle/ga_oracle.c`` -- a plain-C restatement of the reference's CPU path
  (the WFA trace/score kernels, the SW trace/score kernels and the result
  semantics of src/api/api.cpp), built to ``oracle/_build/libga_oracle.so``.
* this module -- the batch-level rules of src/api/api.cpp on top of it:
  request validation and its error strings (api.cpp:246-266, 515-536,
  600-616), the batch smax = minimum (api.cpp:271-272), "any with_cigar puts
  the whole batch on the trace path" (api.cpp:273-274, 621-622), buffer sizing
  (api.cpp:316-320, 636-647) and the resolved/unresolved counters
  (api.cpp:493-496, 843-845).

Parity is pinned: tests/test_oracle.py checks this oracle against
tests/golden/, which was produced by the reference's own kernels compiled for
the host (oracle/ref_wrap.cpp, tests/golden/make_golden.py).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import time
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libga_oracle.so")
_REF_PATH = os.path.join(_HERE, "_ref", "libgaref.so")

K_MAX_SMAX = 511                     # src/api/api.cpp:227
SW_MAX_TRACE_CELLS = 1 << 26         # include/genoaligner/api.hpp:256
# The reference sizes the score-only SW kernel's shared memory as
# 4 warps * 2*(max_n+1) ints (sw_kernel.hip:189-197) and refuses the batch when
# that exceeds the per-block limit the runtime reports (api.cpp:789-797); on a
# CUDA device that attribute is the 48 KiB default.
SW_SCORE_SMEM_LIMIT = 48 * 1024

WFA_OUT = np.dtype([("score", "<i4"), ("resolved", "<i4"), ("rescore_ok", "<i4"),
                    ("wellformed_ok", "<i4"), ("cigar_off", "<i8"), ("cigar_len", "<i4"),
                    ("pad", "<i4")])
SW_OUT = np.dtype([("score", "<i4"), ("resolved", "<i4"), ("start_i", "<i4"),
                   ("start_j", "<i4"), ("end_i", "<i4"), ("end_j", "<i4"),
                   ("rescore_ok", "<i4"), ("wellformed_ok", "<i4"), ("too_large", "<i4"),
                   ("pad", "<i4"), ("cigar_off", "<i8"), ("cigar_len", "<i4"), ("pad2", "<i4")])

_lib = None


def build(quiet: bool = True) -> str:
    """Compile oracle/ga_oracle.c (make -C oracle).  Returns the .so path."""
    out = subprocess.run(["make", "-C", _HERE, "_build/libga_oracle.so"],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(_LIB_PATH):
            build()
        L = ctypes.CDLL(_LIB_PATH)
        p = ctypes.c_void_p
        i32 = ctypes.c_int32
        L.ora_wfa_batch.argtypes = [i32, p, p, p, p, p, p, i32, i32, i32, p, p, p, i32]
        L.ora_wfa_batch.restype = ctypes.c_int
        L.ora_sw_batch.argtypes = [i32, p, p, p, p, p, p, i32, i32, i32, i32, i32, p,
                                   ctypes.c_longlong, i32, p, p, p, i32]
        L.ora_sw_batch.restype = ctypes.c_int
        L.ora_edit_distance_batch.argtypes = [i32, p, p, p, p, p, p, p, i32]
        L.ora_edit_distance_batch.restype = ctypes.c_int
        ip = ctypes.POINTER(ctypes.c_int)
        L.ora_wfa_validate.argtypes = [ctypes.c_char_p, i32, i32, ctypes.c_char_p, i32, ctypes.c_char_p, i32, ip, ip]
        L.ora_wfa_validate.restype = None
        L.ora_sw_validate.argtypes = [ctypes.c_char_p, i32, ctypes.c_char_p, i32, i32, i32, ctypes.c_char_p, i32,
                                      i32, i32, _OraScoring, i32, ip, ip]
        L.ora_sw_validate.restype = None
        _lib = L
    return _lib


class _OraScoring(ctypes.Structure):
    _fields_ = [("match", ctypes.c_int), ("mismatch", ctypes.c_int), ("gap_open", ctypes.c_int),
                ("gap_extend", ctypes.c_int)]


def wfa_validate(cigar: bytes, score: int, pattern: bytes, text: bytes):
    """(rescore_ok, wellformed_ok) of one WFA CIGAR (validate, src/api/api.cpp:84-106)."""
    rs, wf = ctypes.c_int(0), ctypes.c_int(0)
    lib().ora_wfa_validate(cigar, len(cigar), score, pattern, len(pattern), text, len(text), ctypes.byref(rs),
                           ctypes.byref(wf))
    return bool(rs.value), bool(wf.value)


def sw_validate(cigar: bytes, text: bytes, si: int, ei: int, pattern: bytes, sj: int, ej: int, scoring, score: int):
    """(rescore_ok, wellformed_ok) of one SW CIGAR over its span (sw_validate,
    src/api/api.cpp:114-156)."""
    rs, wf = ctypes.c_int(0), ctypes.c_int(0)
    lib().ora_sw_validate(cigar, len(cigar), text, len(text), si, ei, pattern, len(pattern), sj, ej,
                          _OraScoring(*scoring), score, ctypes.byref(rs), ctypes.byref(wf))
    return bool(rs.value), bool(wf.value)


def _ptr(a: np.ndarray):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def pack(seqs):
    """Concatenate byte sequences; returns (buffer, int64 offsets, int32 lengths)."""
    lens = np.fromiter((len(s) for s in seqs), dtype=np.int32, count=len(seqs))
    offs = np.zeros(len(seqs), dtype=np.int64)
    if len(seqs) > 1:
        np.cumsum(lens[:-1], out=offs[1:])
    buf = np.frombuffer(b"".join(seqs) + b"\0" * 8, dtype=np.uint8)
    return buf, offs, lens


@dataclass
class WfaBatch:
    """API-level result of one align_batch call (arrays indexed by request)."""
    status: str = "ok"                 # ok | invalid_argument | device_error
    error: str | None = None
    score: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    resolved: np.ndarray = field(default_factory=lambda: np.zeros(0, bool))
    rescore_ok: np.ndarray = field(default_factory=lambda: np.zeros(0, bool))
    wellformed_ok: np.ndarray = field(default_factory=lambda: np.zeros(0, bool))
    cigars: list = field(default_factory=list)
    resolved_count: int = 0
    unresolved_count: int = 0
    seconds: float = 0.0               # wall time of the C restatement's call alone


@dataclass
class SwBatch:
    status: str = "ok"
    error: str | None = None
    score: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    resolved: np.ndarray = field(default_factory=lambda: np.zeros(0, bool))
    start_i: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    start_j: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    end_i: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    end_j: np.ndarray = field(default_factory=lambda: np.zeros(0, np.int32))
    rescore_ok: np.ndarray = field(default_factory=lambda: np.zeros(0, bool))
    wellformed_ok: np.ndarray = field(default_factory=lambda: np.zeros(0, bool))
    too_large: np.ndarray = field(default_factory=lambda: np.zeros(0, bool))
    cigars: list = field(default_factory=list)
    resolved_count: int = 0
    unresolved_count: int = 0
    seconds: float = 0.0               # wall time of the C restatement's call alone


def _default_wfa(n, status, error):
    b = WfaBatch(status=status, error=error)
    b.score = np.full(n, -1, np.int32)
    b.resolved = np.zeros(n, bool)
    b.rescore_ok = np.zeros(n, bool)
    b.wellformed_ok = np.zeros(n, bool)
    b.cigars = [b""] * n
    return b


def wfa_batch(patterns, texts, smax=64, with_cigar=True, threads=None,
              max_smax=K_MAX_SMAX) -> WfaBatch:
    """align_batch over (pattern, text) byte strings.

    ``smax`` and ``with_cigar`` are scalars or per-request sequences.  A request
    whose pattern/text is ``None`` with a non-zero length is represented by
    passing ``(None, length)`` tuples.  ``max_smax`` is the accepted upper bound
    (511 for the drop-in API; larger for the extension entry)."""
    n = len(patterns)
    smaxs = np.full(n, smax, np.int64) if np.isscalar(smax) else np.asarray(smax, np.int64)
    wants = np.full(n, bool(with_cigar)) if np.isscalar(with_cigar) else np.asarray(with_cigar, bool)
    if n == 0:
        return _default_wfa(0, "ok", None)
    pats, txts = [], []
    for i in range(n):
        p, t = patterns[i], texts[i]
        # null pointer with a non-zero length (api.cpp:248-253)
        if (isinstance(p, tuple) and p[1] > 0) or (isinstance(t, tuple) and t[1] > 0):
            return _default_wfa(n, "invalid_argument", "null pointer with non-zero length")
        if isinstance(p, tuple) and p[1] < 0 or isinstance(t, tuple) and t[1] < 0:
            return _default_wfa(n, "invalid_argument", "negative length")
        if smaxs[i] < 0 or smaxs[i] > max_smax:
            return _default_wfa(n, "invalid_argument",
                                "smax out of range [0, 511]" if max_smax == K_MAX_SMAX
                                else "smax out of range")
        pats.append(b"" if isinstance(p, tuple) else bytes(p))
        txts.append(b"" if isinstance(t, tuple) else bytes(t))
    bsmax = int(smaxs.min())
    trace = bool(wants.any())
    pbuf, poff, plen = pack(pats)
    tbuf, toff, tlen = pack(txts)
    cap = int(max(1, int((plen.astype(np.int64) + tlen + 2).max())))
    cig_len_cap = plen.astype(np.int64) + tlen + 2
    cig_off = np.zeros(n, np.int64)
    if n > 1:
        np.cumsum(cig_len_cap[:-1], out=cig_off[1:])
    cigbuf = np.zeros(int(cig_len_cap.sum()) + 8, np.uint8)
    out = np.zeros(n, WFA_OUT)
    L = lib()
    t0 = time.perf_counter()
    rc = L.ora_wfa_batch(n, _ptr(pbuf), _ptr(poff), _ptr(plen), _ptr(tbuf), _ptr(toff),
                         _ptr(tlen), bsmax, int(trace), cap, _ptr(cigbuf), _ptr(cig_off),
                         _ptr(out), threads or os.cpu_count() or 1)
    t1 = time.perf_counter()
    if rc != 0:
        raise MemoryError("oracle worker allocation failed")
    b = WfaBatch()
    b.seconds = t1 - t0
    b.score = out["score"].copy()
    b.resolved = out["resolved"].astype(bool)
    b.rescore_ok = out["rescore_ok"].astype(bool)
    b.wellformed_ok = out["wellformed_ok"].astype(bool)
    raw = cigbuf.tobytes()
    b.cigars = [raw[o:o + l] for o, l in zip(out["cigar_off"].tolist(), out["cigar_len"].tolist())]
    b.resolved_count = int(b.resolved.sum())
    b.unresolved_count = n - b.resolved_count
    return b


def _default_sw(n, status, error):
    b = SwBatch(status=status, error=error)
    b.score = np.full(n, -1, np.int32)
    for f in ("start_i", "start_j", "end_i", "end_j"):
        setattr(b, f, np.full(n, -1, np.int32))
    b.resolved = np.zeros(n, bool)
    b.rescore_ok = np.zeros(n, bool)
    b.wellformed_ok = np.zeros(n, bool)
    b.too_large = np.zeros(n, bool)
    b.cigars = [b""] * n
    return b


def sw_scheme_error(match, mismatch, gap_open, gap_extend, with_cigar):
    """The refusals of sw_scheme_ok (src/api/api.cpp:515-536), same strings."""
    if match <= 0:
        return "SW scoring: match must be > 0 (the score is 0 for every input otherwise)"
    if mismatch >= match:
        return "SW scoring: mismatch must be < match"
    if gap_open <= 0 or gap_extend <= 0:
        return "SW scoring: gap costs must be > 0"
    if with_cigar and gap_extend > gap_open:
        return ("SW scoring: gap_extend > gap_open with with_cigar cannot re-score "
                "to its own score (api.hpp; RESULTADO_H9_SW2_TRACE.md). Score-only "
                "requests may use it")
    return None


def sw_batch(texts, patterns, scoring=(2, -3, 5, 2), with_cigar=True, threads=None,
             trace_cell_limit=SW_MAX_TRACE_CELLS, score_smem_limit=SW_SCORE_SMEM_LIMIT) -> SwBatch:
    """align_sw_batch over (text, pattern) byte strings; text is the row axis.

    ``scoring`` is one (match, mismatch, gap_open, gap_extend) tuple or a list
    with one per request.  ``trace_cell_limit`` is the per-pair direction-table
    limit (2^26 in the drop-in API).  ``score_smem_limit`` bounds the
    score-only path's pattern length as the reference does (None disables)."""
    n = len(texts)
    if n == 0:
        return _default_sw(0, "ok", None)
    schemes = [tuple(scoring)] * n if np.isscalar(scoring[0]) else [tuple(s) for s in scoring]
    wants = np.full(n, bool(with_cigar)) if np.isscalar(with_cigar) else np.asarray(with_cigar, bool)
    ts, ps = [], []
    for i in range(n):
        t, p = texts[i], patterns[i]
        if (isinstance(t, tuple) and t[1] > 0) or (isinstance(p, tuple) and p[1] > 0):
            return _default_sw(n, "invalid_argument", "null pointer with non-zero length")
        if isinstance(t, tuple) and t[1] < 0 or isinstance(p, tuple) and p[1] < 0:
            return _default_sw(n, "invalid_argument", "negative length")
        err = sw_scheme_error(*schemes[i], bool(wants[i]))
        if err:
            return _default_sw(n, "invalid_argument", err)
        if schemes[i] != schemes[0]:
            return _default_sw(n, "invalid_argument",
                               "all requests in an SW batch must share one scoring scheme")
        ts.append(b"" if isinstance(t, tuple) else bytes(t))
        ps.append(b"" if isinstance(p, tuple) else bytes(p))
    tbuf, toff, tlen = pack(ts)
    pbuf, poff, plen = pack(ps)
    trace = bool(wants.any())
    max_n = int(plen.max())
    max_m = int(tlen.max())
    if not trace and score_smem_limit is not None:
        if 4 * 2 * (max_n + 1) * 4 > score_smem_limit:
            return _default_sw(n, "invalid_argument",
                               "pattern_len exceeds this device's shared-memory limit "
                               "for the score kernel (see api.hpp supported-size limits)")
    max_cells = int(((tlen.astype(np.int64) + 1) * (plen.astype(np.int64) + 1)).max())
    dir_limit = max_cells if trace_cell_limit is None or trace_cell_limit < 0 else min(max_cells, int(trace_cell_limit))
    cap = max_m + max_n + 4
    per = tlen.astype(np.int64) + plen + 4
    cig_off = np.zeros(n, np.int64)
    if n > 1:
        np.cumsum(per[:-1], out=cig_off[1:])
    cigbuf = np.zeros(int(per.sum()) + 8, np.uint8)
    out = np.zeros(n, SW_OUT)
    m_, x_, go, ge = schemes[0]
    want_u8 = wants.astype(np.uint8)            # must outlive the call below
    L = lib()
    t0 = time.perf_counter()
    rc = L.ora_sw_batch(n, _ptr(tbuf), _ptr(toff), _ptr(tlen), _ptr(pbuf), _ptr(poff),
                        _ptr(plen), m_, x_, go, ge, int(trace),
                        _ptr(want_u8), dir_limit, cap, _ptr(cigbuf),
                        _ptr(cig_off), _ptr(out), threads or os.cpu_count() or 1)
    t1 = time.perf_counter()
    if rc != 0:
        raise MemoryError("oracle worker allocation failed")
    b = SwBatch()
    b.seconds = t1 - t0
    for f in ("score", "start_i", "start_j", "end_i", "end_j"):
        setattr(b, f, out[f].copy())
    for f in ("resolved", "rescore_ok", "wellformed_ok", "too_large"):
        setattr(b, f, out[f].astype(bool))
    raw = cigbuf.tobytes()
    b.cigars = [raw[o:o + l] for o, l in zip(out["cigar_off"].tolist(), out["cigar_len"].tolist())]
    b.resolved_count = int(b.resolved.sum())
    b.unresolved_count = n - b.resolved_count
    return b


def edit_distance(patterns, texts, threads=1, timing=False):
    """Levenshtein distances by the O(mn) DP (src/reference/edit_distance_cpu.hpp).
    With timing=True returns (distances, seconds of the C call alone)."""
    n = len(patterns)
    pbuf, poff, plen = pack([bytes(p) for p in patterns])
    tbuf, toff, tlen = pack([bytes(t) for t in texts])
    out = np.zeros(n, np.int32)
    L = lib()
    t0 = time.perf_counter()
    L.ora_edit_distance_batch(n, _ptr(pbuf), _ptr(poff), _ptr(plen), _ptr(tbuf),
                              _ptr(toff), _ptr(tlen), _ptr(out), int(threads or 1))
    t1 = time.perf_counter()
    return (out, t1 - t0) if timing else out
