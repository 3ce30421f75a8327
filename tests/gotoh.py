"""An independent affine-gap local Smith-Waterman (Gotoh, 1982), written from the
published recurrences and not from the reference or the oracle.

TEST INFRASTRUCTURE ONLY: a second opinion on the rescue semantics.  The oracle
restates the reference's kernels (ksw's striped SIMD order, the suboptimal
tracker, the reverse start-recovery pass); this module shares none of that code.
It fills the whole DP matrix of one pair row by row with numpy:

    E(i, j) = max(H(i-1, j) - (o_del + e_del), E(i-1, j) - e_del)       gap in the query
    G(i, j) = max(0, H(i-1, j-1) + s(t_i, q_j), E(i, j))
    F(i, j) = max_{k < j} G(i, k) - o_ins - (j - k) * e_ins             gap in the target
    H(i, j) = max(G(i, j), F(i, j))

Rows i run over the target, columns j over the query (a gap of length n costs
o + n * e, the ksw convention).  Opening F from G rather than from H is exact
for o_ins >= 0: an F-derived H(i, k) opening a new gap never beats extending
the F that produced it, so F is one running prefix maximum per row.

From the matrix, with the end and second-best conventions stated by bwa's
ksw_align2 documentation (mate rescue):
  * score: the maximum of H; te: the first target row holding it; qe: the first
    query column of that row holding it (-1, -1 when score is 0);
  * tb, qb: the start of a best alignment ending at (te, qe), found as the end of
    the same DP run on the reversed prefixes q[..=qe], t[..=te] -- the first
    reversed row reaching score and its first column -- i.e. the shortest best
    alignment ending there;
  * score2, te2: bwa's peak-collapsing recipe over the per-row maxima (rows
    reaching minsc start a peak, a row right after a peak's row replaces it only
    when strictly higher), then the best peak whose row lies more than
    ceil(score / max_sc) rows from te (-1, -1 when none).
"""
from __future__ import annotations

import numpy as np

NEG = -(1 << 40)


def local_matrix(q, t, mat, o_del, e_del, o_ins, e_ins, m=5):
    """H as an int64 array of shape (len(t), len(q))."""
    q = np.asarray(q, dtype=np.int64)
    t = np.asarray(t, dtype=np.int64)
    mat = np.asarray(mat, dtype=np.int64).reshape(m, m)
    ql, tl = len(q), len(t)
    H = np.zeros((tl, ql), dtype=np.int64)
    if ql == 0 or tl == 0:
        return H
    cols = np.arange(ql, dtype=np.int64)
    h_up = np.zeros(ql, dtype=np.int64)   # H(i-1, j), row -1 is all zero
    e_up = np.full(ql, NEG, dtype=np.int64)
    for i in range(tl):
        s = mat[t[i], q]                 # s(t_i, q_j), matrix indexed [target][query]
        diag = np.empty(ql, dtype=np.int64)
        diag[0] = 0                      # H(i-1, -1) = 0
        diag[1:] = h_up[:-1]
        diag += s
        e = np.maximum(h_up - (o_del + e_del), e_up - e_del)
        g = np.maximum(np.maximum(diag, e), 0)
        # F(i, j) = max_{k<j} (G(i, k) + k e) - o - j e
        pre = np.maximum.accumulate(g + cols * e_ins)
        f = np.full(ql, NEG, dtype=np.int64)
        f[1:] = pre[:-1] - o_ins - cols[1:] * e_ins
        h = np.maximum(g, f)
        H[i] = h
        h_up, e_up = h, e
    return H


def _first_max(H, score):
    """(row, column) of the first cell (row-major) holding score, or (-1, -1)."""
    if score <= 0:
        return -1, -1
    rows = np.nonzero(H.max(axis=1) == score)[0]
    r = int(rows[0])
    c = int(np.nonzero(H[r] == score)[0][0])
    return r, c


def peaks_score2(rowmax, score, te, max_sc, minsc):
    """bwa's second-best recipe on the per-row maxima."""
    peaks = []  # [score, row]
    for i, v in enumerate(int(x) for x in rowmax):
        if v < minsc:
            continue
        if peaks and peaks[-1][1] + 1 == i:
            if v > peaks[-1][0]:
                peaks[-1] = [v, i]
        else:
            peaks.append([v, i])
    if score <= 0 or not peaks:
        return -1, -1
    hw = (score + max_sc - 1) // max_sc
    s2, t2 = -1, -1
    for v, r in peaks:
        if (r < te - hw or r > te + hw) and v > s2:
            s2, t2 = v, r
    return s2, t2


def align(q, t, mat, o, e, minsc, max_sc, m=5):
    """(score, qb, qe, tb, te, score2, te2) for symmetric gap costs o, e.
    qb = tb = -1 when score < minsc (bwa runs its start recovery only then)."""
    q = list(q)
    t = list(t)
    H = local_matrix(q, t, mat, o, e, o, e, m)
    score = int(H.max()) if H.size else 0
    te, qe = _first_max(H, score)
    rowmax = H.max(axis=1) if H.size else np.zeros(len(t), dtype=np.int64)
    score2, te2 = peaks_score2(rowmax, score, te, max_sc, minsc)
    qb = tb = -1
    if score >= minsc and qe >= 0:
        R = local_matrix(q[:qe + 1][::-1], t[:te + 1][::-1], mat, o, e, o, e, m)
        rr, rc = _first_max(R, score)
        if rr >= 0:
            tb, qb = te - rr, qe - rc
    return score, qb, qe, tb, te, score2, te2
