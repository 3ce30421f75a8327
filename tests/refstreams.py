"""Bit-for-bit replays of the input streams the reference's own tests draw.

Each generator reproduces the fixed-seed LCG (or xorshift) sequence of one
reference test, in the same draw order, so the parity tests run the exact
cases the reference runs.  Only inputs are reproduced; expected outputs come
from the oracle (and, for the known-answer tests, from the reference's
asserted constants).
"""
from __future__ import annotations

M64 = (1 << 64) - 1
LCG_MUL = 6364136223846793005  # crates/bwa-extend/src/lib.rs:62
LCG_INC = 1442695040888963407  # crates/bwa-extend/src/lib.rs:64


class Lcg:
    """state = state * MUL + INC (wrapping); output state >> 33."""

    def __init__(self, seed):
        self.s = seed & M64

    def __call__(self):
        self.s = (self.s * LCG_MUL + LCG_INC) & M64
        return self.s >> 33


def scmat(a, b):
    m = [-1] * 25
    for r in range(4):
        for c in range(4):
            m[r * 5 + c] = a if r == c else -b
    return m


def backend_matches_scalar():
    """crates/bwa-extend/src/lib.rs:283-354 -- 2000 single extensions, scoring swept.
    Yields dicts with q, t, w, zdrop, end_bonus, h0, a, b, o_del, e_del, o_ins, e_ins."""
    nx = Lcg(0x9E3779B97F4A7C15)
    for case in range(2000):
        qlen = 1 + nx() % 60
        tlen = 1 + nx() % 60
        q = [nx() % 4 for _ in range(qlen)]
        t = [nx() % 4 for _ in range(tlen)]
        w = 1 + nx() % 30
        zdrop = nx() % 120
        end_bonus = nx() % 10
        h0 = 1 + nx() % 20
        if case == 0:
            a, b, od, ed, oi, ei = 1, 4, 6, 1, 6, 1
        else:
            a = 1 + nx() % 4
            b = 1 + nx() % 6
            od = 1 + nx() % 8
            ed = 1 + nx() % 3
            oi = 1 + nx() % 8
            ei = 1 + nx() % 3
        yield dict(q=q, t=t, w=w, zdrop=zdrop, end_bonus=end_bonus, h0=h0, a=a, b=b, o_del=od, e_del=ed,
                   o_ins=oi, e_ins=ei)


def backend_batch_matches_scalar():
    """crates/bwa-extend/src/lib.rs:426-525 -- 200 batches (lane cross-talk)."""
    nx = Lcg(0x123456789ABCDEF0)
    sizes = [1, 2, 3, 4, 7, 8, 9, 15, 16, 17, 20, 31]
    for _ in range(200):
        bs = sizes[nx() % 12]
        w = 1 + nx() % 30
        zdrop = nx() % 120
        end_bonus = nx() % 10
        od = 4 + nx() % 4
        ed = 1 + nx() % 2
        oi = 4 + nx() % 4
        ei = 1 + nx() % 2
        qs = []
        for _ in range(bs):
            ql = 1 + nx() % 80
            qs.append([nx() % 4 for _ in range(ql)])
        ts = []
        for _ in range(bs):
            tl = 1 + nx() % 80
            ts.append([nx() % 4 for _ in range(tl)])
        h0s = [1 + nx() % 20 for _ in range(bs)]
        yield dict(qs=qs, ts=ts, h0s=h0s, w=w, zdrop=zdrop, end_bonus=end_bonus, a=1, b=4, o_del=od,
                   e_del=ed, o_ins=oi, e_ins=ei)


def _mutated_target(nx, q, tlen, keep_per100):
    t = []
    qi = 0
    while len(t) < tlen:
        if qi < len(q) and nx() % 100 >= keep_per100:
            t.append(q[qi])
            qi += 1
        else:
            t.append(nx() % 4)
            if nx() % 2 == 0:
                qi += 1
    return t


def read_sized():
    """crates/bwa-neon/src/lib.rs:279-415 -- 120 read-sized batches (q 60..259)."""
    nx = Lcg(0xC0FFEE123456789A)
    sizes = [1, 5, 8, 9, 16, 17, 24, 40]
    for _ in range(120):
        bs = sizes[nx() % 8]
        w = 50 + nx() % 120
        zdrop = nx() % 200
        end_bonus = nx() % 12
        od = 4 + nx() % 4
        ed = 1 + nx() % 2
        oi = 4 + nx() % 4
        ei = 1 + nx() % 2
        qs, ts, h0s = [], [], []
        for _ in range(bs):
            ql = 60 + nx() % 200
            q = [nx() % 4 for _ in range(ql)]
            tl = ql + nx() % 60
            t = _mutated_target(nx, q, tl, 4)
            qs.append(q)
            ts.append(t)
            h0s.append(20 + nx() % 30)
        yield dict(qs=qs, ts=ts, h0s=h0s, w=w, zdrop=zdrop, end_bonus=end_bonus, a=1, b=4, o_del=od,
                   e_del=ed, o_ins=oi, e_ins=ei)


def ungapped():
    """crates/bwa-neon/src/lib.rs:421-559 -- 300 batches of near-diagonal jobs, N injected."""
    nx = Lcg(0x51ED5EEDD1A60000)
    sizes = [1, 4, 8, 13, 16, 24]
    for _ in range(300):
        bs = sizes[nx() % 6]
        w = 1 + nx() % 150
        zdrop = nx() % 200
        end_bonus = nx() % 12
        qs, ts, h0s = [], [], []
        for _ in range(bs):
            ql = 1 + nx() % 200
            q = [nx() % 4 for _ in range(ql)]
            mode = nx() % 5
            extra = nx() % 40
            t = list(q)
            if mode == 0:
                t.extend(nx() % 4 for _ in range(extra))
            elif mode == 1:
                pass
            elif mode == 2:
                cut = max(ql - (1 + nx() % 3), 0)
                t = t[:cut]
                t.extend(nx() % 4 for _ in range(extra))
            elif mode == 3:
                for _ in range(1 + nx() % 2):
                    if t:
                        p = nx() % len(t)
                        t[p] = (t[p] + 1 + nx() % 3) % 4
                t.extend(nx() % 4 for _ in range(extra))
            else:
                if t:
                    p = nx() % len(t)
                    t[p] = 4
                t.extend(nx() % 4 for _ in range(extra))
            qs.append(q)
            ts.append(t)
            h0s.append(1 + nx() % 40)
        yield dict(qs=qs, ts=ts, h0s=h0s, w=w, zdrop=zdrop, end_bonus=end_bonus, a=1, b=4, o_del=6, e_del=1,
                   o_ins=6, e_ins=1)


def simd_verify():
    """crates/bwa-neon/src/batched.rs:2433-2530 -- u8 (q 1..90) and i16 (q 200..599) kernel sweeps."""
    nx = Lcg(0xA7C2000000000001)
    sizes = [1, 8, 16, 17, 32, 33, 48]
    for _ in range(200):
        w = 1 + nx() % 150
        zdrop = nx() % 200
        end_bonus = nx() % 12
        bs = sizes[nx() % 7]
        for big in (False, True):
            qs, ts, h0s = [], [], []
            for _ in range(bs):
                ql = 200 + nx() % 400 if big else 1 + nx() % 90
                q = [nx() % 4 for _ in range(ql)]
                tl = ql + nx() % 30
                t = _mutated_target(nx, q, tl, 5)
                qs.append(q)
                ts.append(t)
                h0s.append(1 + nx() % 20)
            yield dict(qs=qs, ts=ts, h0s=h0s, w=w, zdrop=zdrop, end_bonus=end_bonus, a=1, b=4, o_del=6,
                       e_del=1, o_ins=6, e_ins=1, big=big)


def unbanded_cases():
    """crates/bwa-extend/src/sw.rs:1326-1356 -- 500 xorshift cases for the unbanded cross-check."""
    M = M64
    st = [0xA5A5123499990001]

    def nxt():
        s = st[0]
        s ^= (s << 13) & M
        s ^= s >> 7
        s ^= (s << 17) & M
        st[0] = s
        return s

    for _ in range(500):
        ln = 20 + nxt() % 40
        base = [nxt() % 4 for _ in range(ln)]
        target = list(base)
        if ln > 25:
            p = ln - 3 - nxt() % 3
            target[p] = (target[p] + 1) % 4
        yield base, target


def matesw_jobs():
    """crates/bwa-neon/src/matesw.rs:5045-5110 -- 2000 rescue jobs (q 5..150, N drawn, planted copies)."""
    nx = Lcg(0x123456789ABCDEF1)
    out = []
    for _ in range(2000):
        ql = 5 + nx() % 146
        tl = ql + nx() % 500
        t = [nx() % 5 for _ in range(tl)]
        q = [nx() % 5 for _ in range(ql)]
        copies = 1 + nx() % 2
        if nx() % 5 != 0:
            for _ in range(copies):
                if tl > ql:
                    at = nx() % (tl - ql + 1)
                    t[at:at + ql] = q
            for _ in range(nx() % 4):
                p = nx() % ql
                q[p] = nx() % 4
        if nx() % 4 == 0:
            q[nx() % ql] = 4
        if nx() % 4 == 0:
            t[nx() % tl] = 4
        out.append((q, t))
    return out


def matesw_pad_columns():
    """crates/bwa-neon/src/matesw.rs:5159-5229 -- 32 jobs, qlen 147 (padded to 160), ragged tlen."""
    nx = Lcg(0xFEEDFACE12345678)
    out = []
    for k in range(1, 33):
        tl = 200 + k * 90
        t = [nx() % 5 for _ in range(tl)]
        q = [nx() % 5 for _ in range(147)]
        t[tl - 147:] = q
        out.append((q, t))
    return out


def matesw_ragged():
    """crates/bwa-neon/src/matesw.rs:5233-5323 -- 32 jobs, tlen 100..3200, endsc 60."""
    nx = Lcg(0x0BADC0DEDEADBEEF)
    out = []
    for k in range(1, 33):
        tl = k * 100
        ql = min(40 + nx() % 111, tl // 2)
        t = [nx() % 5 for _ in range(tl)]
        q = [nx() % 5 for _ in range(ql)]
        at = tl - ql - nx() % 20
        t[at:at + ql] = q
        out.append((q, t))
    return out


def rescue_bench_jobs(n):
    """crates/bwa-neon/src/matesw.rs:4905-4935 -- 150 bp query planted in a 500 bp window."""
    nx = Lcg(0xDEADBEEF12345678)
    out = []
    for _ in range(n):
        t = [nx() % 5 for _ in range(500)]
        q = [nx() % 5 for _ in range(150)]
        at = nx() % (500 - 150 + 1)
        t[at:at + 150] = q
        for _ in range(3):
            p = nx() % 150
            q[p] = nx() % 4
        out.append((q, t))
    return out


def third_party_oracle_pairs():
    """crates/bwa-extend/tests/third_party_oracle.rs:246-298 -- 300 local-SW pairs per scoring:
    qlen 1..160 over the full alphabet (N at ~3%), the target a noisy relative of the query
    (8% substitutions / indels, N injected), tlen = qlen + 0..199.  One stream per scoring,
    restarted from the same seed for each of (1, 4, 6, 1) and (2, 3, 5, 2)."""
    nx = Lcg(0x51D39CF10BADC0DE)
    out = []
    for _ in range(300):
        qlen = 1 + nx() % 160
        q = [4 if nx() % 100 < 3 else nx() % 4 for _ in range(qlen)]
        tlen = qlen + nx() % 200
        t = []
        qi = 0
        while len(t) < tlen:
            if qi < len(q) and nx() % 100 >= 8:
                t.append(q[qi])
                qi += 1
            elif nx() % 100 < 3:
                t.append(4)
                if nx() % 2 == 0:
                    qi += 1
            else:
                t.append(nx() % 4)
                if nx() % 2 == 0:
                    qi += 1
        out.append((q, t))
    return out
