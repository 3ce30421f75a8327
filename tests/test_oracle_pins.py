"""Pins the CPU oracle to the reference before it is trusted as the checker.

The reference (Rust) cannot be built here, so the oracle is pinned by
  * every known-answer test of the reference's own unit tests, with the
    reference's asserted constants, and
  * the cross-form equalities the reference's tests assert, replayed on the
    reference's own input streams: the lockstep extension equals the scalar
    one, the ungapped closed form equals the DP when it fires, the unbanded
    extension equals the banded one where band and z-drop are inactive, and
    the batched (truncated) ksw_align2 equals the scalar one.
"""
import numpy as np
import pytest

import oracle
import refstreams as R

pytestmark = pytest.mark.usefixtures("built")


def test_ksw_align2_kat_perfect_match():
    # crates/bwa-extend/src/sw.rs:1214-1223
    q = [0, 1, 2, 3, 0, 1, 2, 3]
    r = oracle.align2_scalar(q, q, oracle.scmat(1, 4), 6, 1, 6, 1, 4, 1, 16)
    assert r[0] == 8 and (r[1], r[2]) == (0, 7) and (r[3], r[4]) == (0, 7)
    assert oracle.align2_batched(q, q, oracle.scmat(1, 4), 6, 1, 6, 1, 4, 1) == r


def test_ksw_align2_kat_local_trims_flanks():
    # crates/bwa-extend/src/sw.rs:1225-1237
    q = [3, 3, 0, 0, 1, 1, 3, 3]
    t = [2, 0, 0, 1, 1, 2]
    r = oracle.align2_scalar(q, t, oracle.scmat(1, 4), 6, 1, 6, 1, 1, 1, 16)
    assert r[0] == 4 and (r[1], r[2]) == (2, 5) and (r[3], r[4]) == (1, 4)


def test_extend_kat_exact_match():
    # crates/bwa-extend/src/sw.rs:1313-1323
    s = [0, 1, 2, 3] * 4
    r = oracle.extend2(s, s, 1, oracle.scmat(1, 4), 6, 1, 6, 1, 100, 0, 100)
    assert r[0] == 1 + len(s) and r[1] == len(s) and r[2] == len(s) and r[4] == 1 + len(s)


def test_extend_kat_zdrop():
    # crates/bwa-extend/src/sw.rs:1383-1393
    q = [0] * 10 + [1] * 40
    t = [0] * 10 + [2] * 40
    r = oracle.extend2(q, t, 1, oracle.scmat(1, 4), 6, 1, 6, 1, 100, 0, 100)
    assert r[0] == 11 and r[2] == 10


def test_extend_matches_unbanded_reference():
    # crates/bwa-extend/src/sw.rs:1326-1356 (500 xorshift cases, band and z-drop inactive)
    mat = oracle.scmat(1, 4)
    for base, target in R.unbanded_cases():
        got = oracle.extend2(base, target, 1, mat, 6, 1, 6, 1, 1000, 0, 1_000_000)
        assert got[0] == oracle.ref_extend(base, target, 1, mat, 6, 1, 6, 1)


def test_lockstep_equals_scalar_on_gate_stream():
    # crates/bwa-extend/src/lib.rs:283-354 asserts backend == ksw_extend2 over this stream.
    for c in R.backend_matches_scalar():
        mat = oracle.scmat(c["a"], c["b"])
        g = dict(o_del=c["o_del"], e_del=c["e_del"], o_ins=c["o_ins"], e_ins=c["e_ins"], w=c["w"],
                 end_bonus=c["end_bonus"], zdrop=c["zdrop"])
        want = oracle.extend2(c["q"], c["t"], c["h0"], mat, **g)
        got = oracle.extend_lockstep([(c["q"], c["t"], c["h0"])], mat, **g, lanes=1)[0]
        assert got == want


@pytest.mark.parametrize("stream", ["batch", "read_sized", "simd_verify"])
def test_lockstep_equals_scalar_on_batch_streams(stream):
    gen = {"batch": R.backend_batch_matches_scalar, "read_sized": R.read_sized, "simd_verify": R.simd_verify}[stream]
    for k, c in enumerate(gen()):
        if stream == "simd_verify" and k >= 60:
            break
        mat = oracle.scmat(c["a"], c["b"])
        g = dict(o_del=c["o_del"], e_del=c["e_del"], o_ins=c["o_ins"], e_ins=c["e_ins"], w=c["w"],
                 end_bonus=c["end_bonus"], zdrop=c["zdrop"])
        jobs = list(zip(c["qs"], c["ts"], c["h0s"]))
        got = oracle.extend_lockstep(jobs, mat, **g, lanes=8)
        for (q, t, h0), r in zip(jobs, got):
            assert r == oracle.extend2(q, t, h0, mat, **g)


def test_ungapped_hit_equals_dp():
    # crates/bwa-neon/src/lib.rs:421-559: the closed form, when it fires, equals ksw_extend2.
    mat = oracle.scmat(1, 4)
    xt = oracle.x_threshold(1, 4, 6, 1, 6, 1)
    hits = 0
    for c in R.ungapped():
        for q, t, h0 in zip(c["qs"], c["ts"], c["h0s"]):
            hit = oracle.ungapped_hit(q, t, h0, 1, 4, xt, c["zdrop"])
            if hit is not None:
                hits += 1
                assert hit == oracle.extend2(q, t, h0, mat, 6, 1, 6, 1, c["w"], c["end_bonus"], c["zdrop"])
    assert hits > 500


@pytest.mark.parametrize("a,b,minsc", [(1, 4, 19), (10, 40, 190)])
def test_batched_align2_equals_scalar(a, b, minsc):
    # crates/bwa-neon/src/matesw.rs:5045-5139 asserts batched_ksw_align2 == ksw_align2 on this stream.
    mat = oracle.scmat(a, b)
    for q, t in R.matesw_jobs():
        lanes = 16 if len(q) * a < 250 else 8
        want = oracle.align2_scalar(q, t, mat, 6, 1, 6, 1, minsc, a, lanes)
        assert oracle.align2_batched(q, t, mat, 6, 1, 6, 1, minsc, a) == want


def test_padded_qlen_rule():
    # crates/bwa-neon/src/matesw.rs:676-686 and the assertion at :5167
    assert oracle.padded_qlen(147, 1) == 160
    assert oracle.padded_qlen(150, 1) == 160
    assert oracle.padded_qlen(250, 1) == 256
    assert oracle.padded_qlen(25, 10) == 32
    assert oracle.padded_qlen(0, 1) == 0


def test_pad_columns_feed_score2():
    # crates/bwa-neon/src/matesw.rs:5224-5228: the stream populates score2 on >= 8 jobs.
    rs = [oracle.local_fwd(q, t, oracle.scmat(1, 4), 6, 1, 6, 1, 19, oracle.INT_MAX, 1, 16)
          for q, t in R.matesw_pad_columns()]
    assert sum(1 for r in rs if r[3] >= 0) >= 8


def test_extension_bins_threshold():
    # crates/bwa-neon/src/batched.rs:817-865 with default scoring: headroom = 4 + 1.
    mat = oracle.scmat(1, 4)
    assert oracle.ext_bin(100, 200, 150, mat) == 0   # 150 + 100 + 5 = 255 < 256
    assert oracle.ext_bin(101, 200, 150, mat) == 1   # 256
    assert oracle.ext_bin(255, 255, 0 + 1, mat) == 1
    assert oracle.ext_bin(100, 256, 10, mat) == 1    # tlen >= 256
    assert oracle.ext_bin(40000, 100, 10, mat) == 2
    odd = mat.copy()
    odd[6] = 2  # non-uniform matrix -> scalar path
    assert oracle.ext_bin(10, 10, 10, odd) == 2


def test_qlen_zero_convention():
    # crates/bwa-neon/src/batched.rs:1025-1039: score h0, gtle 1, gscore max(h0-o_del-e_del, 0).
    assert oracle.extend2([], [1, 2, 3], 10) == (10, 0, 0, 1, 3, 0)
    assert oracle.extend2([], [1, 2, 3], 5) == (5, 0, 0, 1, 0, 0)
    assert oracle.extend2([], [], 5) == (5, 0, 0, 0, -1, 0)
    assert oracle.extend_lockstep([([], [1, 2, 3], 10)]) == [(10, 0, 0, 1, 3, 0)]


def test_band_clamp_truncates_toward_zero():
    # (qlen*max + end_bonus - o)/e + 1 in double, truncated; floor 1.
    assert oracle.clamp_band(100, 50, 1, 5, 6, 1, 6, 1) == 50
    assert oracle.clamp_band(100, 0, 1, 0, 6, 1, 6, 1) == 1
    assert oracle.clamp_band(100, 10, 1, 0, 6, 4, 6, 1) == 2   # (10-6)/4+1 = 2
    assert oracle.clamp_band(100, 3, 1, 0, 6, 4, 6, 1) == 1    # (3-6)/4+1 = 0.25 -> 0 -> 1


# ---------------------------------------------------------------- ksw_global2

def test_global2_kat_exact_match_is_all_m():
    # crates/bwa-extend/src/sw.rs:1358-1365
    s = [0, 1, 2, 3, 0, 1, 2, 3, 0, 1]
    assert oracle.global2(s, s, 100) == (len(s), [len(s) << 4])


def test_global2_kat_single_deletion():
    # crates/bwa-extend/src/sw.rs:1367-1380
    q = [0, 1, 2, 3, 0, 1, 2, 3]
    t = q[:4] + [2] + q[4:]
    _, cig = oracle.global2(q, t, 100)
    assert sum(c >> 4 for c in cig if c & 0xf == 2) == 1
    assert sum(c >> 4 for c in cig if c & 0xf == 0) == len(q)


def _gotoh_global(q, t, mat, o_del, e_del, o_ins, e_ins, m=5):
    """Textbook unbanded global affine-gap score (independent of the reference's code), with gaps
    opened from the match state as ksw does; small inputs only."""
    NEG = -(1 << 40)
    Q, T = len(q), len(t)
    M = [[NEG] * (Q + 1) for _ in range(T + 1)]
    E = [[NEG] * (Q + 1) for _ in range(T + 1)]  # deletion: consumes target
    F = [[NEG] * (Q + 1) for _ in range(T + 1)]  # insertion: consumes query
    M[0][0] = 0
    for j in range(1, Q + 1):
        F[0][j] = -(o_ins + e_ins * j)
    for i in range(1, T + 1):
        E[i][0] = -(o_del + e_del * i)
    for i in range(1, T + 1):
        for j in range(1, Q + 1):
            best_prev = max(M[i - 1][j - 1], E[i - 1][j - 1], F[i - 1][j - 1])
            M[i][j] = best_prev + mat[t[i - 1] * m + q[j - 1]]
            E[i][j] = max(M[i - 1][j] - o_del - e_del, E[i - 1][j] - e_del)
            F[i][j] = max(M[i][j - 1] - o_ins - e_ins, F[i][j - 1] - e_ins)
    return max(M[T][Q], E[T][Q], F[T][Q])


def _cigar_score(q, t, cig, mat, o_del, e_del, o_ins, e_ins, m=5):
    i = j = 0
    s = 0
    for c in cig:
        op, ln = c & 0xf, c >> 4
        if op == 0:
            for _ in range(ln):
                s += int(mat[t[i] * m + q[j]])
                i += 1
                j += 1
        elif op == 1:
            s -= o_ins + e_ins * ln
            j += ln
        else:
            s -= o_del + e_del * ln
            i += ln
    assert (i, j) == (len(t), len(q))
    return s


def test_global2_against_textbook_and_own_cigar():
    # wide band: the score equals an independent unbanded global DP; in any band where the path
    # stays inside, re-scoring the returned CIGAR gives the returned score
    rng = np.random.default_rng(3)
    mat = oracle.scmat(1, 4)
    for k in range(120):
        t = rng.integers(0, 5 if k % 7 == 0 else 4, int(rng.integers(0, 40))).tolist()
        q = list(t)
        for _ in range(int(rng.integers(0, 4))):  # substitutions and short indels
            if not q:
                break
            p = int(rng.integers(0, len(q)))
            r = rng.random()
            if r < 0.5:
                q[p] = int(rng.integers(0, 4))
            elif r < 0.75:
                del q[p:p + int(rng.integers(1, 3))]
            else:
                q[p:p] = rng.integers(0, 4, int(rng.integers(1, 3))).tolist()
        wide = max(len(q), len(t)) + 1
        score, cig = oracle.global2(q, t, wide, mat)
        assert score == _gotoh_global(q, t, mat, 6, 1, 6, 1), (q, t)
        assert _cigar_score(q, t, cig, mat, 6, 1, 6, 1) == score
        w = abs(len(t) - len(q)) + 3  # the caller's narrowest band, crates/bwa-mem/src/cigar.rs:438-445
        r = oracle.global2(q, t, w, mat)
        assert r is not None
        if len(q) and len(t):
            assert _cigar_score(q, t, r[1], mat, 6, 1, 6, 1) == r[0]


def test_global2_edge_conventions():
    # empty query: the whole target is one leading deletion; empty target: the traceback's
    # leftover column count min(w, qlen) becomes the insertion (sw.rs:726-733)
    assert oracle.global2([], [1, 2, 3], 5) == (-9, [3 << 4 | 2])
    assert oracle.global2([1, 2, 3], [], 2) == (-0x40000000, [2 << 4 | 1])
    assert oracle.global2([], [], 3) == (0, [])


# ---------------------------------------------------------------- rescue windows

def test_pac_unpack_definition():
    # crates/bwa-index/src/fmindex.rs:1170-1190 builds this 64-base .pac (bytes i*37+11) and checks
    # the range unpack against the per-base definition; the oracle is that definition
    pac = np.array([(i * 37 + 11) & 0xff for i in range(17)], dtype=np.uint8)
    l_pac = 64
    fwd = [(int(pac[p >> 2]) >> ((3 - (p & 3)) * 2)) & 3 for p in range(l_pac)]
    want = fwd + [3 - fwd[2 * l_pac - 1 - p] for p in range(l_pac, 2 * l_pac)]
    got = [oracle.lib().ko_ref_base(pac.ctypes.data_as(oracle.C.POINTER(oracle.C.c_uint8)), l_pac, p)
           for p in range(2 * l_pac)]
    assert got == want


def test_rescue_window_rules():
    ref = oracle.Reference(np.zeros(1000, np.uint8), [600, 400])  # contigs [0, 600), [600, 1000)
    L2 = 2000
    # FR (r = 1): reverse, larger: [a + lo - l_ms, a + hi)
    assert oracle.rescue_window(ref, 100, 0, 1, 100, 400, 150, 19) == (True, 50, 500, 0)
    # FF (r = 0): forward, larger: [a + lo, a + hi + l_ms) = [400, 850); its midpoint 625 lies in
    # contig 1, so the window clamps to contig 1 and the anchor's contig 0 does not match
    assert oracle.rescue_window(ref, 300, 0, 0, 100, 400, 150, 19) == (False, 600, 850, 1)
    assert oracle.rescue_window(ref, 300, 1, 0, 100, 400, 150, 19) == (True, 600, 850, 1)
    # RR (r = 3): forward orientation, smaller: [a - hi, a - lo + l_ms), clamped at 0
    assert oracle.rescue_window(ref, 150, 0, 3, 100, 400, 150, 19) == (True, 0, 200, 0)
    # reverse half: [1600, 2050) clipped to 2 * l_pac; midpoint 1800 mirrors to forward 199
    # (contig 0), whose span mirrors to [2000 - 600, 2000) = [1400, 2000)
    assert oracle.rescue_window(ref, 1500, 0, 0, 100, 400, 150, 19) == (True, 1600, 2000, 0)
    # midpoint 1425 mirrors to 574 (contig 0): [1400, 2000) clamps [1200, 1650) to [1400, 1650)
    assert oracle.rescue_window(ref, 1100, 1, 0, 100, 400, 150, 19) == (False, 1400, 1650, 0)
    # too short after the clamp
    assert oracle.rescue_window(ref, 590, 0, 2, 5, 8, 10, 19)[0] is False
    # window entirely outside [0, 2 * l_pac)
    ok, rb, re, rid = oracle.rescue_window(ref, L2 + 500, 1, 0, 100, 400, 150, 19)
    assert not ok and rid == -1
