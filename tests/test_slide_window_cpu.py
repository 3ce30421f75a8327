"""The window argument of the thread-per-job long-query kernel (csrc/ext_slide.cu), checked on
the CPU against ksw_extend2's own row-by-row band (crates/bwa-extend/src/sw.rs:203-493).

The kernel keeps a job's DP row in a window of wc = ceil8(2w + 5 + K) columns (plus two spare
pair words) that moves right K columns before row i whenever i - w - 1 - base >= K.  Its results
equal the full row's if (1) every column a row touches lies in the window it holds, and (2) every
column a row writes lies in [base, base + wc): then a column entering the window on the right has
never been written and holds its row -1 value, as the reference's full row does.  A row touches
at most columns [beg - 1, end + 3] (the odd first column's pair word, the look-ahead pair and
query word) and writes [beg, end] (its cells and the sentinel), beg and end as the reference
computes them.  This test restates ksw_extend2 in Python with its eh row, pins it to the oracle
on every case, and checks both conditions on every row of every case, for the kernel's slide step
(64) and for smaller ones that move the window every few rows."""
import numpy as np
import pytest

import oracle


def extend_rows(q, t, h0, mat, m, o_del, e_del, o_ins, e_ins, w, end_bonus, zdrop, on_row):
    """ksw_extend2 (sw.rs:203-493) over lists of codes; on_row(i, beg, end, clamped w) before each
    row's cells.
    Returns (score, qle, tle, gtle, gscore, max_off)."""
    qlen, tlen = len(q), len(t)
    oe_del, oe_ins = o_del + e_del, o_ins + e_ins
    eh_h = [0] * (qlen + 1)
    eh_e = [0] * (qlen + 1)
    eh_h[0] = h0
    if qlen >= 1:
        eh_h[1] = h0 - oe_ins if h0 > oe_ins else 0
    j = 2
    while j <= qlen and eh_h[j - 1] > e_ins:
        eh_h[j] = eh_h[j - 1] - e_ins
        j += 1
    w = oracle.clamp_band(w, qlen, int(max(mat)), end_bonus, o_ins, e_ins, o_del, e_del)
    best, best_i, best_j, best_ie, gscore, max_off = h0, -1, -1, -1, -1, 0
    beg, end = 0, qlen
    for i in range(tlen):
        f = 0
        rmax, mj = 0, -1
        row = t[i] * m
        beg = max(beg, i - w)
        end = min(end, i + w + 1, qlen)
        h1 = max(h0 - (o_del + e_del * (i + 1)), 0) if beg == 0 else 0
        on_row(i, beg, end, w)
        for j in range(beg, end):
            M, e = eh_h[j], eh_e[j]
            eh_h[j] = h1
            M = M + int(mat[row + q[j]]) if M else 0
            h = max(M, e, f)
            h1 = h
            if rmax <= h:
                mj, rmax = j, h
            e = max(e - e_del, M - oe_del, 0)
            eh_e[j] = e
            f = max(f - e_ins, M - oe_ins, 0)
        eh_h[end], eh_e[end] = h1, 0
        if max(beg, end) == qlen and gscore <= h1:
            best_ie, gscore = i, h1
        if rmax == 0:
            break
        if rmax > best:
            best, best_i, best_j = rmax, i, mj
            max_off = max(max_off, abs(mj - i))
        elif zdrop > 0:
            if i - best_i > mj - best_j:
                if best - rmax - ((i - best_i) - (mj - best_j)) * e_del > zdrop:
                    break
            elif best - rmax - ((mj - best_j) - (i - best_i)) * e_ins > zdrop:
                break
        j = beg
        while j < end and eh_h[j] == 0 and eh_e[j] == 0:
            j += 1
        beg = j
        j = end
        while j >= beg and eh_h[j] == 0 and eh_e[j] == 0:
            j -= 1
        end = j + 2 if j + 2 < qlen else qlen
    return best, best_j + 1, best_i + 1, best_ie + 1, gscore, max_off


class Window:
    """The kernel's window over one job: base, the move rule and the two conditions."""

    def __init__(self, qlen, k, wc):
        self.k, self.wc = k, wc
        self.moves = qlen + 4 > wc
        self.base = 0
        self.moved = 0

    def row(self, i, beg, end, w):
        if self.moves and i - w - 1 - self.base >= self.k:
            self.base += self.k
            self.moved += 1
        if beg >= end:  # an empty row ends the job before anything reads its sentinel
            return
        lo_touch, hi_touch = beg - (beg & 1), end + 3
        assert lo_touch >= self.base, (i, beg, end, self.base)
        assert hi_touch < self.base + self.wc + 4, (i, beg, end, self.base, self.wc)
        assert beg >= self.base and end < self.base + self.wc, (i, beg, end, self.base, self.wc)


def window_cols(w, k):
    return (2 * w + 5 + k + 7) & ~7


def _mutate(rng, t, ql, sub):
    q = list(t[:ql])
    out = []
    for x in q:
        r = rng.random()
        if r < sub:
            out.append(int((x + rng.integers(1, 4)) % 4))
        elif r < sub * 1.1:
            continue  # deletion from the query
        elif r < sub * 1.2:
            out.extend(int(c) for c in rng.integers(0, 4, int(rng.integers(1, 4))))
            out.append(int(x))
        else:
            out.append(int(x))
    return out


def _cases(seed, n):
    rng = np.random.default_rng(seed)
    for _ in range(n):
        ql = int(rng.integers(40, 330))
        tl = max(1, ql + int(rng.integers(-60, 120)))
        t = [int(c) for c in rng.integers(0, 4, tl)]
        kind = int(rng.integers(0, 4))
        if kind == 0:
            q = [int(c) for c in rng.integers(0, 4, ql)]  # unrelated: the band dies early
        else:
            q = _mutate(rng, t + [int(c) for c in rng.integers(0, 4, 400)], ql, (0.01, 0.05, 0.15)[kind - 1])
        for arr in (q, t):
            for x in rng.integers(0, len(arr), int(rng.integers(0, 3))):
                arr[int(x)] = 4  # N
        h0 = int(rng.choice([1, 5, 20, 60, 150, 400]))
        w = int(rng.choice([1, 2, 5, 13, 40]))
        zdrop = int(rng.choice([0, 30, 100]))
        yield q, t, h0, w, zdrop


@pytest.mark.parametrize("k", [8, 16, 64])
def test_window_holds_every_row(k):
    mat = oracle.scmat()
    moved = 0
    for q, t, h0, w, zdrop in _cases(100 + k, 200):
        wclamp = oracle.clamp_band(w, len(q), 1, 5, 6, 1, 6, 1)
        win = Window(len(q), k, window_cols(wclamp, k))
        got = extend_rows(q, t, h0, mat, 5, 6, 1, 6, 1, w, 5, zdrop, win.row)
        want = oracle.extend2(np.array(q, np.uint8), np.array(t, np.uint8), h0, mat, w=w, zdrop=zdrop)
        assert got == tuple(want), (got, want, len(q), len(t), h0, w, zdrop)
        moved += win.moved
    assert moved > (300 if k < 64 else 60)  # the window did move, many times


def test_window_asymmetric_gaps_and_large_h0():
    mat = oracle.scmat(2, 3)
    for q, t, h0, w, zdrop in _cases(7, 120):
        h0 = h0 * 3
        wclamp = oracle.clamp_band(w, len(q), 2, 0, 4, 3, 5, 2)
        win = Window(len(q), 8, window_cols(wclamp, 8))
        got = extend_rows(q, t, h0, mat, 5, 5, 2, 4, 3, w, 0, zdrop, win.row)
        want = oracle.extend2(np.array(q, np.uint8), np.array(t, np.uint8), h0, mat, o_del=5, e_del=2, o_ins=4,
                              e_ins=3, w=w, end_bonus=0, zdrop=zdrop)
        assert got == tuple(want), (got, want)
