"""ctypes front end of the CPU oracle (``oracle/libksworacle.so``).

TEST INFRASTRUCTURE ONLY.  The oracle is the checker the CUDA kernels are
compared against; only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import it.

The C restatement follows the reference's Rust semantics line for line
(``crates/bwa-extend/src/sw.rs``, ``crates/bwa-neon/src/batched.rs``,
``crates/bwa-neon/src/matesw.rs``); see the citations in ``ksw_oracle.c``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "libksworacle.so")
_lib = None

INT_MAX = 2**31 - 1


class ExtResult(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("score", "qle", "tle", "gtle", "gscore", "max_off")]

    def tuple(self):
        return (self.score, self.qle, self.tle, self.gtle, self.gscore, self.max_off)


class AlnResult(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("score", "qb", "qe", "tb", "te", "score2", "te2")]

    def tuple(self):
        return (self.score, self.qb, self.qe, self.tb, self.te, self.score2, self.te2)


class FwdResult(C.Structure):
    _fields_ = [(n, C.c_int32) for n in ("score", "te", "qe", "score2", "te2")]

    def tuple(self):
        return (self.score, self.te, self.qe, self.score2, self.te2)


EXT_DTYPE = np.dtype([(n, np.int32) for n in ("score", "qle", "tle", "gtle", "gscore", "max_off")])
ALN_DTYPE = np.dtype([(n, np.int32) for n in ("score", "qb", "qe", "tb", "te", "score2", "te2")])
FWD_DTYPE = np.dtype([(n, np.int32) for n in ("score", "te", "qe", "score2", "te2")])


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    src = os.path.join(_HERE, "ksw_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        u8p, i8p, i32p, i64p = (C.POINTER(C.c_uint8), C.POINTER(C.c_int8),
                                C.POINTER(C.c_int32), C.POINTER(C.c_int64))
        I = C.c_int
        L.ko_extend2.restype = ExtResult
        L.ko_extend2.argtypes = [u8p, I, u8p, I, I, i8p, I, I, I, I, I, I, I, I,
                                 C.POINTER(C.c_uint64)]
        L.ko_ref_extend.restype = I
        L.ko_ref_extend.argtypes = [u8p, I, u8p, I, I, i8p, I, I, I, I, I]
        L.ko_ungapped_hit.restype = I
        L.ko_ungapped_hit.argtypes = [u8p, I, u8p, I, I, I, I, I, I, C.POINTER(ExtResult)]
        L.ko_x_threshold.restype = I
        L.ko_x_threshold.argtypes = [I] * 6
        L.ko_ext_bin.restype = I
        L.ko_ext_bin.argtypes = [I, I, I, I, i8p]
        L.ko_padded_qlen.restype = I
        L.ko_padded_qlen.argtypes = [I, I]
        L.ko_rescue_width.restype = I
        L.ko_rescue_width.argtypes = [I, C.POINTER(I), C.POINTER(I), I, i8p, I]
        L.ko_clamp_band.restype = I
        L.ko_clamp_band.argtypes = [I] * 8
        L.ko_local_fwd.restype = FwdResult
        L.ko_local_fwd.argtypes = [u8p, I, u8p, I, I, i8p, I, I, I, I, I, I, I, I]
        L.ko_align2_scalar.restype = AlnResult
        L.ko_align2_scalar.argtypes = [u8p, I, u8p, I, I, i8p, I, I, I, I, I, I, I]
        L.ko_align2_batched.restype = AlnResult
        L.ko_align2_batched.argtypes = [u8p, I, u8p, I, I, i8p, I, I, I, I, I, I]
        L.ko_extend_lockstep.restype = None
        L.ko_extend_lockstep.argtypes = [I, C.POINTER(u8p), C.POINTER(I), C.POINTER(u8p),
                                         C.POINTER(I), C.POINTER(I), I, i8p, I, I, I, I, I, I,
                                         I, I, C.POINTER(ExtResult)]
        L.ko_extend_batch.restype = None
        L.ko_extend_batch.argtypes = [u8p, C.c_int64, i64p, i64p, i32p, i32p, i32p, i32p, I,
                                      i8p, I, I, I, I, I, I, I, C.c_void_p,
                                      C.POINTER(C.c_uint64)]
        L.ko_extend_batch_dispatch.restype = None
        L.ko_extend_batch_dispatch.argtypes = [u8p, C.c_int64, i64p, i64p, i32p, i32p, i32p, i32p, I, i8p, I, I, I,
                                               I, I, I, I, C.c_void_p, C.POINTER(C.c_uint64),
                                               C.POINTER(C.c_uint64)]
        L.ko_align2_batch.restype = None
        L.ko_align2_batch.argtypes = [u8p, C.c_int64, i64p, i64p, i32p, i32p, I, i8p, I, I, I,
                                      I, I, I, I, I, I, C.c_void_p, C.POINTER(C.c_uint64)]
        L.ko_global2.restype = I
        L.ko_global2.argtypes = [u8p, I, u8p, I, I, i8p, I, I, I, I, I, i32p, C.POINTER(C.c_uint32),
                                 C.POINTER(I)]
        L.ko_global2_batch.restype = I
        L.ko_global2_batch.argtypes = [u8p, C.c_int64, i64p, i64p, i32p, i32p, i32p, I, i8p, I, I, I, I, I,
                                       i32p, i64p, C.POINTER(C.c_uint32), i32p]
        L.ko_ref_base.restype = C.c_uint8
        L.ko_ref_base.argtypes = [u8p, C.c_int64, C.c_int64]
        L.ko_rescue_window.restype = I
        L.ko_rescue_window.argtypes = [u8p, C.c_int64, i64p, i32p, C.c_int32, C.c_int64, C.c_int32, I, I, I, I, I,
                                       i64p, i64p, i32p]
        L.ko_local_fwd_batch.restype = None
        L.ko_local_fwd_batch.argtypes = [u8p, C.c_int64, i64p, i64p, i32p, i32p, i32p, i32p, I,
                                         i8p, I, I, I, I, I, I, I, C.c_void_p]
        _lib = L
    return _lib


def _u8(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.uint8))
    if a.size == 0:
        a = np.zeros(1, dtype=np.uint8)[:0]
    return a


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct))


def scmat(a: int = 1, b: int = 4) -> np.ndarray:
    """bwa_fill_scmat (crates/bwa-core/src/opt.rs:445-482)."""
    m = np.full(25, -1, dtype=np.int8)
    for r in range(4):
        for c in range(4):
            m[r * 5 + c] = a if r == c else -b
    return m


def _mat(mat):
    return np.ascontiguousarray(np.asarray(mat, dtype=np.int8))


def extend2(q, t, h0, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, w=100, end_bonus=5,
            zdrop=100, m=5, with_cells=False):
    q, t = _u8(q), _u8(t)
    mat = _mat(scmat() if mat is None else mat)
    cells = C.c_uint64(0)
    r = lib().ko_extend2(_p(q, C.c_uint8), len(q), _p(t, C.c_uint8), len(t), m,
                         _p(mat, C.c_int8), o_del, e_del, o_ins, e_ins, w, end_bonus, zdrop, h0,
                         C.byref(cells)).tuple()
    return (r, cells.value) if with_cells else r


def extend_lockstep(jobs, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, w=100, end_bonus=5,
                    zdrop=100, lanes=8, m=5):
    """jobs: list of (query, target, h0)."""
    n = len(jobs)
    mat = _mat(scmat() if mat is None else mat)
    qs = [_u8(j[0]) for j in jobs]
    ts = [_u8(j[1]) for j in jobs]
    QP = (C.POINTER(C.c_uint8) * max(n, 1))(*[_p(a, C.c_uint8) for a in qs])
    TP = (C.POINTER(C.c_uint8) * max(n, 1))(*[_p(a, C.c_uint8) for a in ts])
    QL = (C.c_int * max(n, 1))(*[len(a) for a in qs])
    TL = (C.c_int * max(n, 1))(*[len(a) for a in ts])
    H0 = (C.c_int * max(n, 1))(*[int(j[2]) for j in jobs])
    out = (ExtResult * max(n, 1))()
    lib().ko_extend_lockstep(n, QP, QL, TP, TL, H0, m, _p(mat, C.c_int8), o_del, e_del, o_ins,
                             e_ins, w, end_bonus, zdrop, lanes, out)
    return [out[k].tuple() for k in range(n)]


def ref_extend(q, t, h0, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, m=5):
    q, t = _u8(q), _u8(t)
    mat = _mat(scmat() if mat is None else mat)
    return lib().ko_ref_extend(_p(q, C.c_uint8), len(q), _p(t, C.c_uint8), len(t), m,
                               _p(mat, C.c_int8), o_del, e_del, o_ins, e_ins, h0)


def x_threshold(a, b, o_del, e_del, o_ins, e_ins):
    return lib().ko_x_threshold(a, b, o_del, e_del, o_ins, e_ins)


def ungapped_hit(q, t, h0, a, b, x_thr, zdrop):
    q, t = _u8(q), _u8(t)
    r = ExtResult()
    ok = lib().ko_ungapped_hit(_p(q, C.c_uint8), len(q), _p(t, C.c_uint8), len(t), h0, a, b,
                               x_thr, zdrop, C.byref(r))
    return r.tuple() if ok else None


def ext_bin(qlen, tlen, h0, mat=None, m=5):
    mat = _mat(scmat() if mat is None else mat)
    return lib().ko_ext_bin(qlen, tlen, h0, m, _p(mat, C.c_int8))


def clamp_band(w, qlen, max_sc, end_bonus, o_ins, e_ins, o_del, e_del):
    return lib().ko_clamp_band(w, qlen, max_sc, end_bonus, o_ins, e_ins, o_del, e_del)


def padded_qlen(qlen, max_sc):
    return lib().ko_padded_qlen(qlen, max_sc)


def rescue_width(qlens, tlens, mat=None, max_sc=1, m=5):
    n = len(qlens)
    mat = _mat(scmat() if mat is None else mat)
    QL = (C.c_int * max(n, 1))(*[int(x) for x in qlens])
    TL = (C.c_int * max(n, 1))(*[int(x) for x in tlens])
    return lib().ko_rescue_width(n, QL, TL, m, _p(mat, C.c_int8), max_sc)


def local_fwd(q, t, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, minsc=19, endsc=INT_MAX,
              max_sc=1, lanes=16, m=5):
    q, t = _u8(q), _u8(t)
    mat = _mat(scmat() if mat is None else mat)
    return lib().ko_local_fwd(_p(q, C.c_uint8), len(q), _p(t, C.c_uint8), len(t), m,
                              _p(mat, C.c_int8), o_del, e_del, o_ins, e_ins, minsc, endsc, max_sc,
                              lanes).tuple()


def align2_scalar(q, t, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, minsc=19, max_sc=1,
                  lanes=16, m=5):
    q, t = _u8(q), _u8(t)
    mat = _mat(scmat() if mat is None else mat)
    return lib().ko_align2_scalar(_p(q, C.c_uint8), len(q), _p(t, C.c_uint8), len(t), m,
                                  _p(mat, C.c_int8), o_del, e_del, o_ins, e_ins, minsc, max_sc,
                                  lanes).tuple()


def align2_batched(q, t, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, minsc=19, max_sc=1, m=5):
    q, t = _u8(q), _u8(t)
    mat = _mat(scmat() if mat is None else mat)
    return lib().ko_align2_batched(_p(q, C.c_uint8), len(q), _p(t, C.c_uint8), len(t), m,
                                   _p(mat, C.c_int8), o_del, e_del, o_ins, e_ins, minsc,
                                   max_sc).tuple()


# ---------------------------------------------------------------- flat batches

def extend_batch(js, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, end_bonus=5, zdrop=100,
                 nthreads=0, m=5):
    """js: a JobSet-like object with seq, q_off, t_off, qlen, tlen, h0, w numpy arrays.
    Returns (structured results, total cells)."""
    mat = _mat(scmat() if mat is None else mat)
    n = len(js.qlen)
    out = np.zeros(n, dtype=EXT_DTYPE)
    cells = C.c_uint64(0)
    seq = _u8(js.seq) if len(js.seq) else np.zeros(1, np.uint8)
    lib().ko_extend_batch(_p(seq, C.c_uint8), n, _p(js.q_off, C.c_int64), _p(js.t_off, C.c_int64),
                          _p(js.qlen, C.c_int32), _p(js.tlen, C.c_int32), _p(js.h0, C.c_int32),
                          _p(js.w, C.c_int32), m, _p(mat, C.c_int8), o_del, e_del, o_ins, e_ins,
                          end_bonus, zdrop, nthreads, out.ctypes.data_as(C.c_void_p),
                          C.byref(cells))
    return out, cells.value


def extend_batch_dispatch(js, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, end_bonus=5, zdrop=100,
                          nthreads=0, m=5):
    """The reference's production flow (ungapped closed form, then the DP) over a JobSet-like
    object.  Returns (structured results, jobs settled by the closed form, DP cells evaluated)."""
    mat = _mat(scmat() if mat is None else mat)
    n = len(js.qlen)
    out = np.zeros(n, dtype=EXT_DTYPE)
    settled, cells = C.c_uint64(0), C.c_uint64(0)
    seq = _u8(js.seq) if len(js.seq) else np.zeros(1, np.uint8)
    lib().ko_extend_batch_dispatch(_p(seq, C.c_uint8), n, _p(js.q_off, C.c_int64), _p(js.t_off, C.c_int64),
                                   _p(js.qlen, C.c_int32), _p(js.tlen, C.c_int32), _p(js.h0, C.c_int32),
                                   _p(js.w, C.c_int32), m, _p(mat, C.c_int8), o_del, e_del, o_ins, e_ins,
                                   end_bonus, zdrop, nthreads, out.ctypes.data_as(C.c_void_p), C.byref(settled),
                                   C.byref(cells))
    return out, settled.value, cells.value


def align2_batch(js, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, minsc=19, max_sc=1, mode=0,
                 lanes=0, nthreads=0, m=5):
    """mode 0 = batched_ksw_align2 semantics, mode 1 = scalar ksw_align2."""
    mat = _mat(scmat() if mat is None else mat)
    n = len(js.qlen)
    out = np.zeros(n, dtype=ALN_DTYPE)
    cells = C.c_uint64(0)
    seq = _u8(js.seq) if len(js.seq) else np.zeros(1, np.uint8)
    lib().ko_align2_batch(_p(seq, C.c_uint8), n, _p(js.q_off, C.c_int64), _p(js.t_off, C.c_int64),
                          _p(js.qlen, C.c_int32), _p(js.tlen, C.c_int32), m, _p(mat, C.c_int8),
                          o_del, e_del, o_ins, e_ins, minsc, max_sc, mode, lanes, nthreads,
                          out.ctypes.data_as(C.c_void_p), C.byref(cells))
    return out, cells.value


def local_fwd_batch(js, minsc, endsc, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, max_sc=1,
                    lanes=0, nthreads=0, m=5):
    mat = _mat(scmat() if mat is None else mat)
    n = len(js.qlen)
    out = np.zeros(n, dtype=FWD_DTYPE)
    minsc = np.ascontiguousarray(np.broadcast_to(np.asarray(minsc, np.int32), (n,)))
    endsc = np.ascontiguousarray(np.broadcast_to(np.asarray(endsc, np.int32), (n,)))
    seq = _u8(js.seq) if len(js.seq) else np.zeros(1, np.uint8)
    lib().ko_local_fwd_batch(_p(seq, C.c_uint8), n, _p(js.q_off, C.c_int64),
                             _p(js.t_off, C.c_int64), _p(js.qlen, C.c_int32),
                             _p(js.tlen, C.c_int32), _p(minsc, C.c_int32), _p(endsc, C.c_int32),
                             m, _p(mat, C.c_int8), o_del, e_del, o_ins, e_ins, max_sc, lanes,
                             nthreads, out.ctypes.data_as(C.c_void_p))
    return out


def global2(q, t, w, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, m=5):
    """ksw_global2 (crates/bwa-extend/src/sw.rs:561-740): (score, cigar words) or None where the
    reference's traceback would index out of range."""
    q, t = _u8(q), _u8(t)
    mat = _mat(scmat() if mat is None else mat)
    cig = np.zeros(len(q) + len(t) + 1, dtype=np.uint32)
    sc, nc = C.c_int32(), C.c_int()
    rc = lib().ko_global2(_p(q, C.c_uint8), len(q), _p(t, C.c_uint8), len(t), m, _p(mat, C.c_int8), o_del, e_del,
                          o_ins, e_ins, w, C.byref(sc), _p(cig, C.c_uint32), C.byref(nc))
    if rc != 0:
        return None
    return int(sc.value), [int(x) for x in cig[:nc.value]]


def global2_batch(js, mat=None, o_del=6, e_del=1, o_ins=6, e_ins=1, nthreads=0, m=5):
    """Every job of a JobSet-like object (per-job w).  Returns (scores, offsets, words): job k's
    CIGAR is words[offsets[k]:offsets[k+1]]; raises if any traceback leaves the matrix."""
    mat = _mat(scmat() if mat is None else mat)
    n = len(js.qlen)
    ql = np.ascontiguousarray(js.qlen, dtype=np.int32)
    tl = np.ascontiguousarray(js.tlen, dtype=np.int32)
    w = np.ascontiguousarray(js.w, dtype=np.int32)
    cap = ql.astype(np.int64) + tl + 1
    cig_off = np.zeros(n, dtype=np.int64)
    if n:
        cig_off[1:] = np.cumsum(cap)[:-1]
    words = np.zeros(int(cap.sum()) + 1, dtype=np.uint32)
    score = np.zeros(n, dtype=np.int32)
    ncig = np.zeros(n, dtype=np.int32)
    qo = np.ascontiguousarray(js.q_off, dtype=np.int64)
    to = np.ascontiguousarray(js.t_off, dtype=np.int64)
    seq = _u8(js.seq) if len(js.seq) else np.zeros(1, np.uint8)
    rc = lib().ko_global2_batch(_p(seq, C.c_uint8), n, _p(qo, C.c_int64), _p(to, C.c_int64), _p(ql, C.c_int32),
                                _p(tl, C.c_int32), _p(w, C.c_int32), m, _p(mat, C.c_int8), o_del, e_del, o_ins,
                                e_ins, nthreads, _p(score, C.c_int32), _p(cig_off, C.c_int64),
                                _p(words, C.c_uint32), _p(ncig, C.c_int32))
    if rc != 0:
        raise ValueError("a traceback left the stored band")
    offsets = np.zeros(n + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(ncig)
    dense = np.zeros(int(offsets[-1]), dtype=np.uint32)
    for k in range(n):
        dense[offsets[k]:offsets[k + 1]] = words[cig_off[k]:cig_off[k] + ncig[k]]
    return score, offsets, dense


class Reference:
    """A 2-bit packed reference (bwa's .pac layout) with its contig table."""

    def __init__(self, bases, contig_lens):
        bases = np.ascontiguousarray(bases, dtype=np.uint8)
        self.l_pac = len(bases)
        pad = (-len(bases)) % 4
        b = np.concatenate([bases, np.zeros(pad, np.uint8)]).reshape(-1, 4)
        self.pac = np.ascontiguousarray((b[:, 0] << 6) | (b[:, 1] << 4) | (b[:, 2] << 2) | b[:, 3], dtype=np.uint8)
        self.len = np.ascontiguousarray(contig_lens, dtype=np.int32)
        self.off = np.zeros(len(self.len), dtype=np.int64)
        self.off[1:] = np.cumsum(self.len.astype(np.int64))[:-1]
        assert int(self.off[-1]) + int(self.len[-1]) == self.l_pac

    def bases(self, rb, re):
        """Bases of [rb, re) in 2*l_pac space (reverse half = reverse complement)."""
        return np.array([lib().ko_ref_base(_p(self.pac, C.c_uint8), self.l_pac, p) for p in range(rb, re)],
                        dtype=np.uint8)


def rescue_window(ref, anchor_rb, anchor_rid, orient, low, high, l_ms, min_seed_len):
    """(valid, rb, re, rid) of one orientation's window (matesw_collect + bns_fetch_seq)."""
    rb, re, rid = C.c_int64(), C.c_int64(), C.c_int32()
    ok = lib().ko_rescue_window(_p(ref.pac, C.c_uint8), ref.l_pac, _p(ref.off, C.c_int64), _p(ref.len, C.c_int32),
                                len(ref.len), anchor_rb, anchor_rid, orient, low, high, l_ms, min_seed_len,
                                C.byref(rb), C.byref(re), C.byref(rid))
    return bool(ok), rb.value, re.value, rid.value


def mate_for_orientation(mate, orient):
    """The query matesw_collect aligns: the mate, reverse-complemented when the orientation is
    reverse (pe.rs:641-648; N stays N)."""
    mate = np.asarray(mate, dtype=np.uint8)
    if (orient >> 1) != (orient & 1):
        return np.where(mate[::-1] < 4, 3 - mate[::-1], 4).astype(np.uint8)
    return mate.copy()
