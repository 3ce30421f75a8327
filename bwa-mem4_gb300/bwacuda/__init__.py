"""Python front end of ``libbwacuda.so`` (ctypes over the C ABI in include/bwacuda.h).

This module is plumbing for tests, the benchmark and Python callers: it lays out
jobs in numpy arrays, calls the C entry points and returns numpy structured
arrays.  All computation happens in the CUDA library; if the library is missing
or no GPU is visible the calls raise instead of falling back to anything else.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_PKG = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(_PKG, "libbwacuda.so")
SYNTH_PATH = os.path.join(_PKG, "libbwasynth.so")

OK, EINVAL, EBASE, ENOMEM, ECUDA, ETIMEOUT, EUNSUPPORTED, EBUSY, EAGAIN, ESHORT = 0, -1, -2, -3, -4, -5, -6, -7, -8, -9
OPT_EXT_PATH, OPT_CHUNK_JOBS, OPT_GRAPHS, OPT_PERSIST_BLOCK, OPT_RESCUE_KERNEL = 1, 2, 3, 4, 5
RESCUE_AUTO, RESCUE_TPJ = 0, 1
OPT_HOST_GATHER = 6
GATHER_AUTO, GATHER_HOST, GATHER_DEVICE = 0, 1, 2
OPT_GRAB, OPT_BUCKET_STEP, OPT_RESCUE_LANES, OPT_UNGAPPED, OPT_DEVICE_PIECE = 7, 8, 9, 10, 11
OPT_LONG_QLEN, OPT_LONG_LANES, OPT_RESCUE_PAIR, OPT_LONG_SLIDE = 12, 13, 14, 15
PATH_PLAIN, PATH_BATCHED = 0, 1
INT_MAX = 2**31 - 1

# ---------------------------------------------------------------- struct layouts (include/bwacuda.h)
EXT_JOB = np.dtype([("query", "u8"), ("target", "u8"), ("qlen", "i4"), ("tlen", "i4"), ("h0", "i4")],
                   align=True)
RES_JOB = np.dtype([("query", "u8"), ("target", "u8"), ("qlen", "i4"), ("tlen", "i4")], align=True)
FWD_JOB = np.dtype([("query", "u8"), ("target", "u8"), ("qlen", "i4"), ("tlen", "i4"), ("minsc", "i4"),
                    ("endsc", "i4")], align=True)
WINDOW_REQ = np.dtype([("mate", "u8"), ("l_ms", "i4"), ("orient", "i4"), ("anchor_rb", "i8"), ("anchor_rid", "i4"),
                       ("low", "i4"), ("high", "i4")], align=True)
WINDOW_RES = np.dtype([("rb", "i8"), ("re", "i8"), ("rid", "i4"), ("valid", "i4")] +
                      [(n, "i4") for n in ("score", "qb", "qe", "tb", "te", "score2", "te2")], align=True)
GLOBAL_JOB = np.dtype([("query", "u8"), ("target", "u8"), ("qlen", "i4"), ("tlen", "i4"), ("w", "i4")],
                      align=True)
DEV_EXT_JOB = np.dtype([("q_off", "u8"), ("t_off", "u8"), ("qlen", "i4"), ("tlen", "i4"), ("h0", "i4"),
                        ("w", "i4")], align=True)
DEV_RES_JOB = np.dtype([("q_off", "u8"), ("t_off", "u8"), ("qlen", "i4"), ("tlen", "i4"), ("minsc", "i4"),
                        ("endsc", "i4")], align=True)
EXT_RES = np.dtype([(n, "i4") for n in ("score", "qle", "tle", "gtle", "gscore", "max_off")])
ALN_RES = np.dtype([(n, "i4") for n in ("score", "qb", "qe", "tb", "te", "score2", "te2")])
FWD_RES = np.dtype([(n, "i4") for n in ("score", "te", "qe", "score2", "te2")])
assert EXT_JOB.itemsize == 32 and RES_JOB.itemsize == 24 and FWD_JOB.itemsize == 32
assert DEV_EXT_JOB.itemsize == 32 and DEV_RES_JOB.itemsize == 32


class Scoring(C.Structure):
    _fields_ = [("m", C.c_int32), ("mat", C.c_int8 * 64), ("o_del", C.c_int32), ("e_del", C.c_int32),
                ("o_ins", C.c_int32), ("e_ins", C.c_int32)]


STAT_FIELDS = ("ext_jobs", "ext_cells", "ext_bin_u8", "ext_bin_i16", "ext_bin_i32", "rescue_jobs",
               "rescue_cells", "rescue_width_u8", "rescue_width_i16", "rescue_width_i32",
               "kernel_launches", "h2d_bytes", "d2h_bytes", "global_jobs", "global_cells", "ext_retry_jobs")


class ServerConfig(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_uint64), ("max_waves", C.c_int32), ("max_requests", C.c_int32)]


class Tuning(C.Structure):
    _fields_ = [("persist_block", C.c_int32), ("grab", C.c_int32), ("bucket_step", C.c_int32),
                ("rescue_lanes", C.c_int32), ("rescue_kernel", C.c_int32), ("candidates", C.c_int32),
                ("ext_gcups", C.c_double), ("rescue_gcups", C.c_double), ("long_qlen", C.c_int32),
                ("long_lanes", C.c_int32), ("rescue_pair", C.c_int32), ("reserved", C.c_int32)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class Stats(C.Structure):
    _fields_ = [(n, C.c_uint64) for n in STAT_FIELDS]


# Every symbol include/bwacuda.h declares.
EXPORTS = ("bwacuda_ctx_create", "bwacuda_ctx_destroy", "bwacuda_set_option", "bwacuda_strerror",
           "bwacuda_backend_name", "bwacuda_extend", "bwacuda_extend_batch", "bwacuda_ksw_align2_batch",
           "bwacuda_ksw_align2_scalar_batch", "bwacuda_ksw_local_fwd_batch", "bwacuda_extend_device",
           "bwacuda_ksw_align2_device", "bwacuda_ctx_sync", "bwacuda_get_stats", "bwacuda_reset_stats",
           "bwacuda_ksw_align2_device_noalloc", "bwacuda_server_start", "bwacuda_server_stop",
           "bwacuda_server_submit_extend", "bwacuda_server_submit_rescue", "bwacuda_server_wait",
           "bwacuda_server_stats", "bwacuda_measure_alu_peak", "bwacuda_get_tuning", "bwacuda_autotune_extend",
           "bwacuda_autotune_rescue", "bwacuda_ksw_global2_batch", "bwacuda_extend_batch_retry",
           "bwacuda_extend_retry_device", "bwacuda_ref_set", "bwacuda_mate_rescue_windows",
           "bwacuda_server_submit_mixed", "bwacuda_server_cells", "bwacuda_measure_op_rate",
           "bwacuda_measure_host_link")

# bwacuda_measure_op_rate operations, in header order
OP_RATE_NAMES = ("viaddmax_s32", "viaddmax_s32_relu", "viaddmax_s16x2", "viaddmax_s16x2_relu", "viaddmin_s16x2",
                 "vimax3_s16x2", "vimax3_u16x2", "vimax_s16x2_relu", "vimax3_s32", "prmt", "c_add_max", "imad",
                 "lop3")

_lib = None
_synth = None


class BwaCudaError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = code
        msg = lib().bwacuda_strerror(code).decode() if _lib is not None else str(code)
        super().__init__(f"{what}: {msg} ({code})")


def lib():
    """Load libbwacuda.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} missing: build it with `python bwa-mem4_gb300/build.py`")
    L = C.CDLL(LIB_PATH)
    vp, I, sz = C.c_void_p, C.c_int, C.c_size_t
    L.bwacuda_ctx_create.argtypes = [I, C.POINTER(vp)]
    L.bwacuda_measure_alu_peak.argtypes = [vp, C.POINTER(C.c_double)]
    L.bwacuda_measure_op_rate.argtypes = [vp, I, C.POINTER(C.c_double)]
    L.bwacuda_measure_host_link.argtypes = [vp, C.c_size_t, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]
    L.bwacuda_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
    L.bwacuda_ksw_global2_batch.argtypes = [vp, vp, sz, I, vp, I, I, I, I, vp, vp, vp, sz]
    L.bwacuda_ref_set.argtypes = [vp, vp, C.c_int64, vp, vp, C.c_int32]
    L.bwacuda_mate_rescue_windows.argtypes = [vp, vp, sz, I, vp, I, I, I, I, I, I, I, vp]
    L.bwacuda_extend_batch_retry.argtypes = [vp, vp, sz, I, vp, I, I, I, I, I, I, I, I, vp, vp, vp]
    L.bwacuda_extend_retry_device.argtypes = [vp, vp, vp, sz, C.POINTER(Scoring), I, I, I, vp, vp, vp, vp]
    L.bwacuda_autotune_extend.argtypes = [vp, vp, vp, sz, C.POINTER(Scoring), I, I, sz, C.POINTER(Tuning)]
    L.bwacuda_autotune_rescue.argtypes = [vp, vp, vp, sz, C.POINTER(Scoring), I, I, sz, C.POINTER(Tuning)]
    L.bwacuda_ctx_destroy.argtypes = [vp]
    L.bwacuda_ctx_destroy.restype = None
    L.bwacuda_set_option.argtypes = [vp, I, C.c_int64]
    L.bwacuda_strerror.argtypes = [I]
    L.bwacuda_strerror.restype = C.c_char_p
    L.bwacuda_backend_name.restype = C.c_char_p
    L.bwacuda_extend.argtypes = [vp, vp, C.c_int32, vp, C.c_int32, I, vp, I, I, I, I, I, I, I, I, vp]
    L.bwacuda_extend_batch.argtypes = [vp, vp, sz, I, vp, I, I, I, I, I, I, I, vp]
    L.bwacuda_ksw_align2_batch.argtypes = [vp, vp, sz, I, vp, I, I, I, I, I, I, vp]
    L.bwacuda_ksw_align2_scalar_batch.argtypes = [vp, vp, sz, I, vp, I, I, I, I, I, I, I, vp]
    L.bwacuda_ksw_local_fwd_batch.argtypes = [vp, vp, sz, I, vp, I, I, I, I, I, I, vp]
    L.bwacuda_extend_device.argtypes = [vp, vp, vp, sz, C.POINTER(Scoring), I, I, I, vp, vp]
    L.bwacuda_ksw_align2_device.argtypes = [vp, vp, vp, sz, C.POINTER(Scoring), I, I, I, I, vp, vp]
    L.bwacuda_ksw_align2_device_noalloc.argtypes = [vp, vp, vp, sz, C.POINTER(Scoring), I, I, I, I, vp, vp]
    L.bwacuda_server_start.argtypes = [vp, C.POINTER(ServerConfig)]
    L.bwacuda_server_stop.argtypes = [vp]
    L.bwacuda_server_submit_extend.argtypes = [vp, vp, sz, C.POINTER(Scoring), I, I, I, C.POINTER(C.c_uint64)]
    L.bwacuda_server_submit_rescue.argtypes = [vp, vp, sz, C.POINTER(Scoring), I, I, C.POINTER(C.c_uint64)]
    L.bwacuda_server_wait.argtypes = [vp, C.c_uint64, vp, C.c_int64, C.POINTER(C.c_int64)]
    L.bwacuda_server_stats.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    L.bwacuda_server_submit_mixed.argtypes = [vp, vp, sz, vp, sz, C.POINTER(Scoring), I, I, I, I, I,
                                              C.POINTER(C.c_uint64)]
    L.bwacuda_server_cells.argtypes = [vp, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    L.bwacuda_ctx_sync.argtypes = [vp]
    L.bwacuda_get_stats.argtypes = [vp, C.POINTER(Stats)]
    L.bwacuda_reset_stats.argtypes = [vp]
    _lib = L
    return L


def synth_lib():
    global _synth
    if _synth is None:
        if not os.path.exists(SYNTH_PATH):
            raise RuntimeError(f"{SYNTH_PATH} missing: build it with `python bwa-mem4_gb300/build.py`")
        S = C.CDLL(SYNTH_PATH)
        u64, i64, vp, I = C.c_uint64, C.c_int64, C.c_void_p, C.c_int
        S.synth_ext1_sizes.argtypes = [u64, i64, vp, vp, vp, vp]
        S.synth_ext1_fill.argtypes = [u64, i64, vp, vp, vp, vp, vp]
        S.synth_ext2_sizes.argtypes = [u64, i64, I, vp, vp, vp, vp]
        S.synth_ext2_fill.argtypes = [u64, i64, I, vp, vp, vp, vp, vp]
        S.synth_res4_sizes.argtypes = [u64, i64, vp, vp]
        S.synth_res4_fill.argtypes = [u64, i64, vp, vp, vp, vp, vp]
        S.synth_glb5_sizes.argtypes = [u64, i64, vp, vp, vp]
        S.synth_glb5_fill.argtypes = [u64, i64, vp, vp, vp, vp, vp]
        _synth = S
    return _synth


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


def scmat(a: int = 1, b: int = 4) -> np.ndarray:
    """bwa_fill_scmat (crates/bwa-core/src/opt.rs:445-482)."""
    m = np.full(25, -1, dtype=np.int8)
    for r in range(4):
        for c in range(4):
            m[r * 5 + c] = a if r == c else -b
    return m


# ---------------------------------------------------------------- job sets

@dataclass
class JobSet:
    """Jobs laid out flat: all bases in ``seq``, per-job byte offsets and lengths."""
    seq: np.ndarray
    q_off: np.ndarray
    t_off: np.ndarray
    qlen: np.ndarray
    tlen: np.ndarray
    h0: np.ndarray
    w: np.ndarray

    def __len__(self):
        return len(self.qlen)

    @staticmethod
    def from_lists(queries, targets, h0=None, w=None) -> "JobSet":
        n = len(queries)
        ql = np.array([len(q) for q in queries], dtype=np.int32)
        tl = np.array([len(t) for t in targets], dtype=np.int32)
        parts = []
        for q, t in zip(queries, targets):
            parts.append(np.asarray(q, dtype=np.uint8))
            parts.append(np.asarray(t, dtype=np.uint8))
        seq = np.concatenate(parts) if parts else np.zeros(0, np.uint8)
        sizes = np.empty(2 * n, dtype=np.int64)
        sizes[0::2] = ql
        sizes[1::2] = tl
        offs = np.concatenate([[0], np.cumsum(sizes)[:-1]]).astype(np.int64) if n else np.zeros(0, np.int64)
        h0a = np.full(n, 1, np.int32) if h0 is None else np.ascontiguousarray(np.broadcast_to(np.asarray(h0, np.int32), (n,)))
        wa = np.full(n, 100, np.int32) if w is None else np.ascontiguousarray(np.broadcast_to(np.asarray(w, np.int32), (n,)))
        return JobSet(seq, offs[0::2].copy(), offs[1::2].copy(), ql, tl, h0a, wa)

    def query(self, k):
        return self.seq[self.q_off[k]:self.q_off[k] + self.qlen[k]]

    def target(self, k):
        return self.seq[self.t_off[k]:self.t_off[k] + self.tlen[k]]

    def head(self, k: int) -> "JobSet":
        """The first k jobs, sharing this set's base buffer."""
        return JobSet(self.seq, self.q_off[:k], self.t_off[:k], self.qlen[:k], self.tlen[:k], self.h0[:k],
                      self.w[:k])

    def take(self, idx) -> "JobSet":
        idx = np.asarray(idx)
        return JobSet.from_lists([self.query(k) for k in idx], [self.target(k) for k in idx],
                                 self.h0[idx], self.w[idx])

    def dev_ext_jobs(self) -> np.ndarray:
        d = np.zeros(len(self), dtype=DEV_EXT_JOB)
        d["q_off"], d["t_off"], d["qlen"], d["tlen"], d["h0"], d["w"] = (
            self.q_off, self.t_off, self.qlen, self.tlen, self.h0, self.w)
        return d

    def dev_res_jobs(self, minsc=0, endsc=0) -> np.ndarray:
        d = np.zeros(len(self), dtype=DEV_RES_JOB)
        d["q_off"], d["t_off"], d["qlen"], d["tlen"] = self.q_off, self.t_off, self.qlen, self.tlen
        d["minsc"], d["endsc"] = minsc, endsc
        return d


def _layout(qlen, tlen):
    sizes = np.empty(2 * len(qlen), dtype=np.int64)
    sizes[0::2] = qlen
    sizes[1::2] = tlen
    offs = np.zeros(len(sizes) + 1, dtype=np.int64)
    np.cumsum(sizes, out=offs[1:])
    return offs[0:-1:2].copy(), offs[1:-1:2].copy(), int(offs[-1])


def synth_ext(config: int, n: int, seed: int = 0) -> JobSet:
    """Extension workloads: 1 = 20k-job style, 2 = 2x150 read pairs, 3 = mixed read lengths / bands."""
    S = synth_lib()
    ql, tl, h0, w = (np.zeros(n, np.int32) for _ in range(4))
    if config == 1:
        S.synth_ext1_sizes(seed, n, _ptr(ql), _ptr(tl), _ptr(h0), _ptr(w))
    else:
        S.synth_ext2_sizes(seed, n, 1 if config == 3 else 0, _ptr(ql), _ptr(tl), _ptr(h0), _ptr(w))
    qo, to, total = _layout(ql, tl)
    seq = np.zeros(max(total, 1), np.uint8)
    if config == 1:
        S.synth_ext1_fill(seed, n, _ptr(qo), _ptr(to), _ptr(ql), _ptr(tl), _ptr(seq))
    else:
        S.synth_ext2_fill(seed, n, 1 if config == 3 else 0, _ptr(qo), _ptr(to), _ptr(ql), _ptr(tl), _ptr(seq))
    return JobSet(seq, qo, to, ql, tl, h0, w)


def synth_rescue(n: int, seed: int = 0) -> JobSet:
    """Mate-rescue workload: 150 bp query vs 750 bp window (10% without the true mate)."""
    S = synth_lib()
    ql, tl = np.zeros(n, np.int32), np.zeros(n, np.int32)
    S.synth_res4_sizes(seed, n, _ptr(ql), _ptr(tl))
    qo, to, total = _layout(ql, tl)
    seq = np.zeros(max(total, 1), np.uint8)
    S.synth_res4_fill(seed, n, _ptr(qo), _ptr(to), _ptr(ql), _ptr(tl), _ptr(seq))
    return JobSet(seq, qo, to, ql, tl, np.ones(n, np.int32), np.zeros(n, np.int32))


def synth_global(n: int, seed: int = 0) -> JobSet:
    """CIGAR-stage workload for ksw_global2: reads of 100/150/250 bp against the reference interval
    they aligned to (1% substitutions, 1-3 bp indels), band per job from bwa-mem's sizing rule."""
    S = synth_lib()
    ql, tl, w = np.zeros(n, np.int32), np.zeros(n, np.int32), np.zeros(n, np.int32)
    S.synth_glb5_sizes(seed, n, _ptr(ql), _ptr(tl), _ptr(w))
    qo, to, total = _layout(ql, tl)
    seq = np.zeros(max(total, 1), np.uint8)
    S.synth_glb5_fill(seed, n, _ptr(qo), _ptr(to), _ptr(ql), _ptr(tl), _ptr(seq))
    return JobSet(seq, qo, to, ql, tl, np.ones(n, np.int32), w)


class RescueWindows:
    """A synthetic genome in bwa's 2-bit .pac layout with its contig table, and mate-rescue
    requests against it: anchors on both strands and all four orientations, insert window
    [low, high], 150 bp mates drawn from inside their window (reverse-complemented where the
    orientation expects it) with 0.5% substitutions, 10% unrelated mates."""

    def __init__(self, n, seed=0, contig_lens=(3_000_000, 1_000_000, 500_000, 2_000_000), low=100, high=700,
                 l_ms=150):
        rng = np.random.default_rng(seed)
        self.contig_lens = np.array(contig_lens, dtype=np.int32)
        self.contig_off = np.zeros(len(contig_lens), dtype=np.int64)
        self.contig_off[1:] = np.cumsum(self.contig_lens.astype(np.int64))[:-1]
        self.l_pac = int(self.contig_lens.sum())
        self.bases = rng.integers(0, 4, self.l_pac).astype(np.uint8)
        pad = (-self.l_pac) % 4
        b = np.concatenate([self.bases, np.zeros(pad, np.uint8)]).reshape(-1, 4)
        self.pac = np.ascontiguousarray((b[:, 0] << 6) | (b[:, 1] << 4) | (b[:, 2] << 2) | b[:, 3], dtype=np.uint8)
        L2 = 2 * self.l_pac
        two = np.concatenate([self.bases, 3 - self.bases[::-1]])  # the 2L text
        # anchors: a contig, a position inside it, a strand
        c = rng.integers(0, len(contig_lens), n)
        pos = self.contig_off[c] + (rng.random(n) * self.contig_lens[c]).astype(np.int64)
        rev = rng.random(n) < 0.5
        self.anchor_rb = np.where(rev, L2 - 1 - pos, pos).astype(np.int64)
        self.anchor_rid = c.astype(np.int32)
        self.orient = rng.integers(0, 4, n).astype(np.int32)
        self.low, self.high = low, high
        # the expected window (before the contig clamp) and a mate from inside it
        is_rev = (self.orient >> 1) != (self.orient & 1)
        larger = (self.orient >> 1) == 0
        a = self.anchor_rb
        rb = np.where(~is_rev, np.where(larger, a + low, a - high), np.where(larger, a + low, a - high) - l_ms)
        re = np.where(~is_rev, np.where(larger, a + high, a - low) + l_ms, np.where(larger, a + high, a - low))
        rb = np.clip(rb, 0, L2)
        re = np.clip(re, 0, L2)
        span = np.maximum(re - rb - l_ms, 0)
        start = rb + (rng.random(n) * (span + 1)).astype(np.int64)
        start = np.clip(start, 0, L2 - l_ms)
        seg = np.lib.stride_tricks.sliding_window_view(two, l_ms)[start]
        mates = np.where(is_rev[:, None], 3 - seg[:, ::-1], seg)
        mut = rng.random((n, l_ms)) < 0.005
        mates = np.where(mut, (mates + 1 + rng.integers(0, 3, (n, l_ms))) & 3, mates)
        unrelated = rng.random(n) < 0.10
        mates[unrelated] = rng.integers(0, 4, (int(unrelated.sum()), l_ms))
        self.mates = np.ascontiguousarray(mates.astype(np.uint8))
        self.l_ms = l_ms
        self.n = n

    def requests(self):
        r = np.zeros(self.n, dtype=WINDOW_REQ)
        r["mate"] = self.mates.ctypes.data + np.arange(self.n, dtype=np.uint64) * self.l_ms
        r["l_ms"] = self.l_ms
        r["orient"] = self.orient
        r["anchor_rb"] = self.anchor_rb
        r["anchor_rid"] = self.anchor_rid
        r["low"], r["high"] = self.low, self.high
        return r


# ---------------------------------------------------------------- context

class Context:
    """One bwacuda_ctx on a CUDA device."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        rc = lib().bwacuda_ctx_create(device, C.byref(h))
        if rc != OK:
            raise BwaCudaError(rc, "bwacuda_ctx_create")
        self.h = h

    def close(self):
        if self.h:
            lib().bwacuda_ctx_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc, what):
        if rc != OK:
            raise BwaCudaError(rc, what)

    def set_option(self, opt, value):
        self._check(lib().bwacuda_set_option(self.h, opt, value), "bwacuda_set_option")

    def stats(self) -> dict:
        s = Stats()
        self._check(lib().bwacuda_get_stats(self.h, C.byref(s)), "bwacuda_get_stats")
        return {n: getattr(s, n) for n in STAT_FIELDS}

    def reset_stats(self):
        self._check(lib().bwacuda_reset_stats(self.h), "bwacuda_reset_stats")

    # -- host-buffer entry points (pointers into js.seq) --
    @staticmethod
    def _host_jobs(js: JobSet, dtype, minsc=None, endsc=None):
        base = js.seq.ctypes.data
        a = np.zeros(len(js), dtype=dtype)
        a["query"] = base + js.q_off.astype(np.uint64)
        a["target"] = base + js.t_off.astype(np.uint64)
        a["qlen"], a["tlen"] = js.qlen, js.tlen
        if "h0" in dtype.names:
            a["h0"] = js.h0
        if "minsc" in dtype.names:
            a["minsc"], a["endsc"] = minsc, endsc
        return a

    def extend_batch(self, js: JobSet, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, w=100, end_bonus=5,
                     zdrop=100, m=5) -> np.ndarray:
        mat = np.ascontiguousarray(scmat() if mat is None else mat, dtype=np.int8)
        jobs = self._host_jobs(js, EXT_JOB)
        out = np.zeros(len(js), dtype=EXT_RES)
        rc = lib().bwacuda_extend_batch(self.h, _ptr(jobs), len(js), m, _ptr(mat), o_del, e_del, o_ins, e_ins,
                                        w, end_bonus, zdrop, _ptr(out))
        self._check(rc, "bwacuda_extend_batch")
        return out

    def extend(self, q, t, h0, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, w=100, end_bonus=5, zdrop=100, m=5):
        mat = np.ascontiguousarray(scmat() if mat is None else mat, dtype=np.int8)
        q = np.ascontiguousarray(q, dtype=np.uint8)
        t = np.ascontiguousarray(t, dtype=np.uint8)
        out = np.zeros(1, dtype=EXT_RES)
        rc = lib().bwacuda_extend(self.h, _ptr(q), len(q), _ptr(t), len(t), m, _ptr(mat), o_del, e_del, o_ins,
                                  e_ins, w, end_bonus, zdrop, h0, _ptr(out))
        self._check(rc, "bwacuda_extend")
        return tuple(int(x) for x in out[0])

    def extend_batch_retry(self, js: JobSet, prev=None, max_tries=2, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1,
                           w=100, end_bonus=5, zdrop=100, m=5):
        """run_side's band-doubling loop: (results, band each job was accepted at)."""
        mat = np.ascontiguousarray(scmat() if mat is None else mat, dtype=np.int8)
        jobs = self._host_jobs(js, EXT_JOB)
        out = np.zeros(len(js), dtype=EXT_RES)
        wu = np.zeros(len(js), dtype=np.int32)
        pv = None if prev is None else np.ascontiguousarray(prev, dtype=np.int32)
        rc = lib().bwacuda_extend_batch_retry(self.h, _ptr(jobs), len(js), m, _ptr(mat), o_del, e_del, o_ins, e_ins,
                                              w, end_bonus, zdrop, max_tries, None if pv is None else _ptr(pv),
                                              _ptr(out), _ptr(wu))
        self._check(rc, "bwacuda_extend_batch_retry")
        return out, wu

    def extend_retry_device(self, d_seq, d_jobs, n, d_out, d_w_used=0, d_prev=0, max_tries=2, sc: Scoring = None,
                            end_bonus=5, zdrop=100, stream=None):
        sc = sc or self.scoring()
        rc = lib().bwacuda_extend_retry_device(self.h, C.c_void_p(d_seq), C.c_void_p(d_jobs), n, C.byref(sc),
                                               end_bonus, zdrop, max_tries, C.c_void_p(d_prev) if d_prev else None,
                                               C.c_void_p(d_out), C.c_void_p(d_w_used) if d_w_used else None,
                                               C.c_void_p(stream) if stream else None)
        self._check(rc, "bwacuda_extend_retry_device")

    def ref_set(self, rw: "RescueWindows"):
        rc = lib().bwacuda_ref_set(self.h, _ptr(rw.pac), rw.l_pac, _ptr(rw.contig_off), _ptr(rw.contig_lens),
                                   len(rw.contig_lens))
        self._check(rc, "bwacuda_ref_set")

    def mate_rescue_windows(self, reqs: np.ndarray, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, minsc=20,
                            max_sc=1, min_seed_len=19, m=5) -> np.ndarray:
        mat = np.ascontiguousarray(scmat() if mat is None else mat, dtype=np.int8)
        out = np.zeros(len(reqs), dtype=WINDOW_RES)
        rc = lib().bwacuda_mate_rescue_windows(self.h, _ptr(reqs), len(reqs), m, _ptr(mat), o_del, e_del, o_ins,
                                               e_ins, minsc, max_sc, min_seed_len, _ptr(out))
        self._check(rc, "bwacuda_mate_rescue_windows")
        return out

    def ksw_global2_batch(self, js: JobSet, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, m=5):
        """ksw_global2 per job (band js.w per job): (scores, offsets, cigar words); job k's CIGAR
        is words[offsets[k]:offsets[k + 1]]."""
        mat = np.ascontiguousarray(scmat() if mat is None else mat, dtype=np.int8)
        n = len(js)
        base = js.seq.ctypes.data
        jobs = np.zeros(n, dtype=GLOBAL_JOB)
        jobs["query"] = base + js.q_off.astype(np.uint64)
        jobs["target"] = base + js.t_off.astype(np.uint64)
        jobs["qlen"], jobs["tlen"], jobs["w"] = js.qlen, js.tlen, js.w
        score = np.zeros(max(n, 1), dtype=np.int32)
        offs = np.zeros(n + 1, dtype=np.uint64)
        cap = int(js.qlen.astype(np.int64).sum() + js.tlen.astype(np.int64).sum()) + 1
        words = np.zeros(cap, dtype=np.uint32)
        rc = lib().bwacuda_ksw_global2_batch(self.h, _ptr(jobs), n, m, _ptr(mat), o_del, e_del, o_ins, e_ins,
                                             _ptr(score), _ptr(offs), _ptr(words), cap)
        self._check(rc, "bwacuda_ksw_global2_batch")
        return score[:n], offs.astype(np.int64), words[:int(offs[-1])]

    def ksw_align2_batch(self, js: JobSet, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, minsc=19, max_sc=1,
                         m=5) -> np.ndarray:
        mat = np.ascontiguousarray(scmat() if mat is None else mat, dtype=np.int8)
        jobs = self._host_jobs(js, RES_JOB)
        out = np.zeros(len(js), dtype=ALN_RES)
        rc = lib().bwacuda_ksw_align2_batch(self.h, _ptr(jobs), len(js), m, _ptr(mat), o_del, e_del, o_ins,
                                            e_ins, minsc, max_sc, _ptr(out))
        self._check(rc, "bwacuda_ksw_align2_batch")
        return out

    def ksw_align2_scalar_batch(self, js: JobSet, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, minsc=19,
                                max_sc=1, lanes=0, m=5) -> np.ndarray:
        mat = np.ascontiguousarray(scmat() if mat is None else mat, dtype=np.int8)
        jobs = self._host_jobs(js, RES_JOB)
        out = np.zeros(len(js), dtype=ALN_RES)
        rc = lib().bwacuda_ksw_align2_scalar_batch(self.h, _ptr(jobs), len(js), m, _ptr(mat), o_del, e_del,
                                                   o_ins, e_ins, minsc, max_sc, lanes, _ptr(out))
        self._check(rc, "bwacuda_ksw_align2_scalar_batch")
        return out

    def ksw_local_fwd_batch(self, js: JobSet, minsc, endsc, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1,
                            max_sc=1, lanes=0, m=5) -> np.ndarray:
        mat = np.ascontiguousarray(scmat() if mat is None else mat, dtype=np.int8)
        jobs = self._host_jobs(js, FWD_JOB, minsc, endsc)
        out = np.zeros(len(js), dtype=FWD_RES)
        rc = lib().bwacuda_ksw_local_fwd_batch(self.h, _ptr(jobs), len(js), m, _ptr(mat), o_del, e_del, o_ins,
                                               e_ins, max_sc, lanes, _ptr(out))
        self._check(rc, "bwacuda_ksw_local_fwd_batch")
        return out

    # -- device-resident entry points (torch tensors or raw device pointers) --
    @staticmethod
    def scoring(mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, m=5) -> Scoring:
        mat = np.asarray(scmat() if mat is None else mat, dtype=np.int8)
        s = Scoring()
        s.m = m
        for k in range(m * m):
            s.mat[k] = int(mat[k])
        s.o_del, s.e_del, s.o_ins, s.e_ins = o_del, e_del, o_ins, e_ins
        return s

    def extend_device(self, d_seq, d_jobs, n, d_out, sc: Scoring = None, end_bonus=5, zdrop=100,
                      path=PATH_BATCHED, stream=None):
        sc = sc or self.scoring()
        rc = lib().bwacuda_extend_device(self.h, C.c_void_p(d_seq), C.c_void_p(d_jobs), n, C.byref(sc),
                                         end_bonus, zdrop, path, C.c_void_p(d_out),
                                         C.c_void_p(stream) if stream else None)
        self._check(rc, "bwacuda_extend_device")

    def ksw_align2_device(self, d_seq, d_jobs, n, d_out, sc: Scoring = None, minsc=19, max_sc=1, mode=0,
                          lanes=0, stream=None):
        sc = sc or self.scoring()
        rc = lib().bwacuda_ksw_align2_device(self.h, C.c_void_p(d_seq), C.c_void_p(d_jobs), n, C.byref(sc),
                                             minsc, max_sc, mode, lanes, C.c_void_p(d_out),
                                             C.c_void_p(stream) if stream else None)
        self._check(rc, "bwacuda_ksw_align2_device")

    def ksw_align2_device_noalloc(self, d_seq, d_jobs, n, d_out, sc: Scoring = None, minsc=19, max_sc=1, mode=0,
                                 lanes=0, stream=None):
        """The allocation-free variant (synchronous); see include/bwacuda.h."""
        sc = sc or self.scoring()
        rc = lib().bwacuda_ksw_align2_device_noalloc(self.h, C.c_void_p(d_seq), C.c_void_p(d_jobs), n, C.byref(sc),
                                                     minsc, max_sc, mode, lanes, C.c_void_p(d_out),
                                                     C.c_void_p(stream) if stream else None)
        self._check(rc, "bwacuda_ksw_align2_device_noalloc")

    # -- serving loop --
    def server_start(self, hbm_budget_bytes=1 << 30, max_waves=3, max_requests=4096):
        cfg = ServerConfig(hbm_budget_bytes, max_waves, max_requests)
        self._check(lib().bwacuda_server_start(self.h, C.byref(cfg)), "bwacuda_server_start")
        self._held = {}

    def server_stop(self):
        self._check(lib().bwacuda_server_stop(self.h), "bwacuda_server_stop")
        self._held = {}

    def submit_extend(self, js: JobSet, sc: Scoring = None, w=100, end_bonus=5, zdrop=100) -> int:
        """Queue an extension request; js must stay alive until wait() (kept here)."""
        jobs = self._host_jobs(js, EXT_JOB)
        rid = C.c_uint64()
        sc = sc or self.scoring()
        rc = lib().bwacuda_server_submit_extend(self.h, _ptr(jobs), len(js), C.byref(sc), w, end_bonus, zdrop,
                                                C.byref(rid))
        self._check(rc, "bwacuda_server_submit_extend")
        self._held[rid.value] = (js, jobs, EXT_RES)
        return rid.value

    def submit_rescue(self, js: JobSet, sc: Scoring = None, minsc=19, max_sc=1) -> int:
        jobs = self._host_jobs(js, RES_JOB)
        rid = C.c_uint64()
        sc = sc or self.scoring()
        rc = lib().bwacuda_server_submit_rescue(self.h, _ptr(jobs), len(js), C.byref(sc), minsc, max_sc,
                                                C.byref(rid))
        self._check(rc, "bwacuda_server_submit_rescue")
        self._held[rid.value] = (js, jobs, ALN_RES)
        return rid.value

    def submit_mixed(self, ejs: JobSet, rjs: JobSet, sc: Scoring = None, w=100, end_bonus=5, zdrop=100, minsc=19,
                     max_sc=1) -> int:
        """Queue one request holding extension jobs ejs and rescue jobs rjs."""
        ejobs = self._host_jobs(ejs, EXT_JOB)
        rjobs = self._host_jobs(rjs, RES_JOB)
        rid = C.c_uint64()
        sc = sc or self.scoring()
        rc = lib().bwacuda_server_submit_mixed(self.h, _ptr(ejobs), len(ejs), _ptr(rjobs), len(rjs), C.byref(sc), w,
                                               end_bonus, zdrop, minsc, max_sc, C.byref(rid))
        self._check(rc, "bwacuda_server_submit_mixed")
        self._held[rid.value] = ((ejs, rjs), (ejobs, rjobs), None)
        return rid.value

    def wait(self, rid, timeout_us=-1):
        """Results of a request and its submit-to-completion latency in seconds (a mixed
        request's results as (extension results, rescue results))."""
        js, jobs, dt = self._held[rid]
        if dt is None:
            ne, nr = len(js[0]), len(js[1])
            raw = np.zeros(ne * EXT_RES.itemsize + nr * ALN_RES.itemsize + 1, dtype=np.uint8)
            out = raw
        else:
            out = np.zeros(len(js), dtype=dt)
        lat = C.c_int64()
        rc = lib().bwacuda_server_wait(self.h, rid, _ptr(out), timeout_us, C.byref(lat))
        if rc == EAGAIN or rc == ETIMEOUT:
            raise BwaCudaError(rc, "bwacuda_server_wait")
        del self._held[rid]
        self._check(rc, "bwacuda_server_wait")
        if dt is None:
            cut = ne * EXT_RES.itemsize
            out = (raw[:cut].view(EXT_RES).copy(), raw[cut:cut + nr * ALN_RES.itemsize].view(ALN_RES).copy())
        return out, lat.value * 1e-9

    def server_cells(self):
        """(extension cells, rescue cells) served since the loop started."""
        a, b = C.c_uint64(), C.c_uint64()
        self._check(lib().bwacuda_server_cells(self.h, C.byref(a), C.byref(b)), "bwacuda_server_cells")
        return a.value, b.value

    def server_stats(self):
        a, b, q = C.c_uint64(), C.c_uint64(), C.c_uint64()
        self._check(lib().bwacuda_server_stats(self.h, C.byref(a), C.byref(b), C.byref(q)), "bwacuda_server_stats")
        return {"served_jobs": a.value, "waves": b.value, "queued": q.value}

    def sync(self):
        self._check(lib().bwacuda_ctx_sync(self.h), "bwacuda_ctx_sync")

    def tuning(self) -> dict:
        t = Tuning()
        self._check(lib().bwacuda_get_tuning(self.h, C.byref(t)), "bwacuda_get_tuning")
        return t.as_dict()

    def autotune_extend(self, d_seq, d_jobs, n, sc: Scoring = None, end_bonus=5, zdrop=100, sample=0) -> dict:
        """Pick the batched extension launch shape on a sample of a device-resident batch."""
        t = Tuning()
        sc = sc or self.scoring()
        rc = lib().bwacuda_autotune_extend(self.h, C.c_void_p(d_seq), C.c_void_p(d_jobs), n, C.byref(sc), end_bonus,
                                           zdrop, sample, C.byref(t))
        self._check(rc, "bwacuda_autotune_extend")
        return t.as_dict()

    def autotune_rescue(self, d_seq, d_jobs, n, sc: Scoring = None, minsc=19, max_sc=1, sample=0) -> dict:
        """Pick the rescue kernel (wavefront lanes per job, or thread-per-job) on a sample."""
        t = Tuning()
        sc = sc or self.scoring()
        rc = lib().bwacuda_autotune_rescue(self.h, C.c_void_p(d_seq), C.c_void_p(d_jobs), n, C.byref(sc), minsc,
                                           max_sc, sample, C.byref(t))
        self._check(rc, "bwacuda_autotune_rescue")
        return t.as_dict()

    def measure_op_rates(self) -> dict:
        """Measured throughput (1e9 lane-operations/s) of each integer operation of the DP kernels."""
        out = {}
        for k, name in enumerate(OP_RATE_NAMES):
            g = C.c_double()
            self._check(lib().bwacuda_measure_op_rate(self.h, k, C.byref(g)), "bwacuda_measure_op_rate")
            out[name] = g.value
        return out

    def measure_host_link(self, nbytes: int = 1 << 30) -> dict:
        """Measured host-link bandwidth (GB/s): device reads of pinned host memory, the copy
        engine's host-to-device copy, device writes to pinned host memory."""
        r, cp, w = C.c_double(), C.c_double(), C.c_double()
        self._check(lib().bwacuda_measure_host_link(self.h, nbytes, C.byref(r), C.byref(cp), C.byref(w)),
                    "bwacuda_measure_host_link")
        return {"device_read_gbs": r.value, "copy_h2d_gbs": cp.value, "device_write_gbs": w.value}

    def measure_alu_peak(self) -> float:
        """Measured integer ALU-pipe rate of the device, 1e9 fused add-max ops per second."""
        g = C.c_double()
        self._check(lib().bwacuda_measure_alu_peak(self.h, C.byref(g)), "bwacuda_measure_alu_peak")
        return g.value
